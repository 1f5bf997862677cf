"""Learned initial guess: a small BF16 3-D CNN predicting the displacement
field from (f, g), trained on the GPU by the package's own kernels
(include/vdvc_cnn.h)."""
