# Recipe that compiles the reference's own C sources, unmodified and where they
# lie, into oracle/_ref/libfdtdref.so (the reference oracle).  Test
# infrastructure only.  The sources are read from REF (default /root/reference);
# nothing is copied into this repository.  The single-rank MPI shim in
# oracle/mpi_stub stands in for an MPI library (none is installed here).
#
#   make -f oracle/ref.mk            # from the repository root
REF     ?= /root/reference
ORACLE  := $(patsubst %/,%,$(dir $(lastword $(MAKEFILE_LIST))))
OUT     := $(ORACLE)/_ref
CC      ?= gcc
# drawer.c is compiled without USE_OPENGL: only its BMP writer remains.
# -std=gnu99 and -DLINUX_OS are what the reference needs (function.c:47 guards
# its directory helpers on LINUX_OS; -std=c99 hides M_PI).  -ffp-contract=off
# keeps the x86 rounding when this is built on an FMA-capable host.
CFLAGS  := -std=gnu99 -O3 -fPIC -ffp-contract=off -DLINUX_OS -w -I$(ORACLE)/mpi_stub -I$(REF)

REF_SRCS := field.c simulator.c noModel.c \
            multiLayerModel.c traceImageModel.c concentricCircleModel.c \
            ntffTM.c ntffTE.c ntff.c cfft.c myComplex.c function.c parser.c drawer.c
HARNESS  := ref_mpi_tm.c ref_mpi_te.c ref_ser_tm.c ref_ser_te.c ref_models.c \
            ref_circle.c ref_morpho.c ref_zigzag.c ref_split_tm.c ref_split_te.c ref_ns_tm.c \
            ref_ns_te.c ref_driver.c

$(OUT)/libfdtdref.so: $(ORACLE)/ref.mk $(addprefix $(REF)/,$(REF_SRCS)) $(addprefix $(ORACLE)/ref_harness/,$(HARNESS)) $(ORACLE)/mpi_stub/mpi.h
	mkdir -p $(OUT)
	$(CC) $(CFLAGS) -shared -o $@ $(addprefix $(REF)/,$(REF_SRCS)) $(addprefix $(ORACLE)/ref_harness/,$(HARNESS)) -lm
