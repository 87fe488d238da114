"""Learned far-field surrogate: training pairs from the batched engine
(data.py) and a small Fourier neural operator with hand-written BF16
tensor-core kernels (model.py, csrc/surrogate_*.cu)."""
