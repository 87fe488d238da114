"""Golden-vector cases: parameters only (shared by make_golden.py and the tests).

Each case is run on the reference's own sources compiled unmodified
(oracle/_ref) by make_golden.py; the outputs are frozen into <name>.npz.

kind "full"  : complete fields / eps on the active cells, NTFF rows for the
               angles in NTFF_ROWS plus per-angle sums and norms of every row.
kind "stats" : per-row sums and norms only (large grids).
Extras: "spectrum" (ntff*_TimeOutput, serial solvers), "frequency"
(ntffTM_Frequency on the final fields), "elliptic" (field_outputElliptic's
file of the final E field) and "image" (drawer_outputImage's BMP of eps).
"""

# FieldInfo order (field.h:20-28): width_nm, height_nm, h_u_nm, pml, lambda_nm, angle_deg, step_num
DISCS_A = [(8.0, 30.0, 7.0, 3.0), (30.0, 32.0, 10.0, 2.25), (50.0, 14.0, 6.0, 4.0), (33.5, 55.0, 5.5, 1.7)]
DISCS_B = [(20.0, 20.0, 9.0, 2.0), (45.0, 40.0, 12.0, 3.5), (58.0, 58.0, 5.0, 1.3)]

CASES = {
    # The 276^2 vacuum run exactly as the reference runs it: every field stays 0.
    "mpi_tm_vacuum_c1": dict(solver="MPI_TM_UPML", fi=(1380, 1380, 5, 10, 400, 0, 2000),
                             model=("none",), steps=2000, kind="stats"),
    "mpi_tm_circle": dict(solver="MPI_TM_UPML", fi=(300, 320, 5, 6, 100, 0, 150),
                          model=("circle", 60, 0.0), steps=150, kind="full",
                          extras=("frequency", "elliptic", "image")),
    "mpi_te_circle": dict(solver="MPI_TE_UPML", fi=(300, 320, 5, 6, 100, 0, 150),
                          model=("circle", 60, 0.0), steps=150, kind="full", extras=("elliptic", "image")),
    "mpi_tm_discs_30deg": dict(solver="MPI_TM_UPML", fi=(310, 300, 5, 7, 80, 30, 140),
                               model=("discs", DISCS_A), steps=140, kind="full"),
    "mpi_te_discs_60deg": dict(solver="MPI_TE_UPML", fi=(300, 310, 5, 7, 80, 60, 140),
                               model=("discs", DISCS_B), steps=140, kind="full"),
    "mpi_tm_morpho": dict(solver="MPI_TM_UPML", fi=(330, 340, 5, 6, 90, 0, 130),
                          model=("morpho", 150, 20, 25, 3, 10, 0.5, 0.0), steps=130, kind="full",
                          extras=("image",)),
    "mpi_te_morpho_eps225": dict(solver="MPI_TE_UPML", fi=(330, 340, 5, 6, 90, 15, 130),
                                 model=("morpho", 150, 20, 25, 3, 0, 0.0, 2.25), steps=130, kind="full"),
    # zigzagModel.c at its first structure (300 nm, 80 nm, 5 layers, 10 deg) and a steeper one
    "mpi_tm_zigzag": dict(solver="MPI_TM_UPML", fi=(500, 600, 5, 8, 100, 0, 120),
                          model=("zigzag", 300, 80, 5, 10), steps=120, kind="full", extras=("image",)),
    "mpi_te_zigzag_40deg": dict(solver="MPI_TE_UPML", fi=(400, 420, 5, 8, 90, 20, 120),
                                model=("zigzag", 200, 50, 3, 40), steps=120, kind="full"),
    "ser_tm_circle": dict(solver="TM_UPML", fi=(300, 300, 5, 8, 100, 0, 700),
                          model=("circle", 60, 0.0), steps=700, kind="full", rows="few",
                          extras=("spectrum", "frequency")),
    "ser_te_circle": dict(solver="TE_UPML", fi=(300, 300, 5, 8, 100, 20, 700),
                          model=("circle", 60, 0.0), steps=700, kind="full", rows="few",
                          extras=("spectrum",)),
    # The split-field PML and NS-FDTD solvers (they have no NTFF: no_ntff).
    "split_tm_circle": dict(solver="TM_2D", fi=(300, 320, 5, 10, 100, 0, 200),
                            model=("circle", 60, 0.0), steps=200, kind="full", no_ntff=True, extras=("elliptic",)),
    "split_te_circle_30deg": dict(solver="TE_2D", fi=(320, 300, 5, 10, 100, 30, 200),
                                  model=("circle", 60, 2.25), steps=200, kind="full", no_ntff=True,
                                  extras=("elliptic",)),
    "ns_tm_morpho": dict(solver="NS_TM_2D", fi=(330, 340, 5, 10, 90, 0, 180),
                         model=("morpho", 150, 20, 25, 3, 10, 0.5, 0.0), steps=180, kind="full", no_ntff=True,
                         extras=("elliptic",)),
    "ns_te_circle_20deg": dict(solver="NS_TE_2D", fi=(300, 320, 5, 10, 100, 20, 200),
                               model=("circle", 60, 0.0), steps=200, kind="full", no_ntff=True,
                               extras=("elliptic",)),
    # The 1044^2 Mie grid (r 500 nm, eps 2.25 override) for the first 40 of 4000 steps.
    "mpi_tm_c2_head": dict(solver="MPI_TM_UPML", fi=(5220, 5220, 5, 10, 500, 0, 4000),
                           model=("circle", 500, 2.25), steps=40, kind="stats"),
    "mpi_te_c2_head": dict(solver="MPI_TE_UPML", fi=(5220, 5220, 5, 10, 500, 0, 4000),
                           model=("circle", 500, 2.25), steps=40, kind="stats"),
}

# NTFF rows stored in full: corners (where the flat index spills into the
# neighbouring angle's row) and a coarse sweep.
NTFF_ROWS = sorted(set(list(range(0, 360, 15)) + [44, 45, 46, 134, 135, 136, 224, 225, 226, 314, 315, 316, 359]))
# long runs keep fewer full rows; their spectrum covers every angle
NTFF_ROWS_FEW = [0, 45, 90, 135, 180, 225, 270, 315, 359]


def make_model(spec):
    """Build an oracle.pyoracle.Model from a case's model tuple."""
    from oracle.pyoracle import Model
    kind = spec[0]
    if kind == "none":
        return Model.none()
    if kind == "circle":
        return Model.circle(spec[1], spec[2])
    if kind == "discs":
        return Model.discs(spec[1])
    if kind == "zigzag":
        return Model.zigzag(*spec[1:5])
    if kind == "morpho":
        w, t0, t1, layers, branch, edge, eps = spec[1:8]
        return Model.morpho(w, t0, t1, layers, branch, edge, eps)
    raise ValueError(kind)
