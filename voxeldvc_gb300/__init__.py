"""voxeldvc_gb300: the voxelDVC global Gauss-Newton DVC path on GB300
(sm_103a), with hand-written CUDA kernels behind a C ABI (include/vdvc.h).

The public modules mirror the reference package's engine API:
``voxeldvc_gb300.engine.geometry_dvc``, ``.kernels_dvc`` and
``.correlate_gpu``, plus the ``voxeldvc run`` driver in ``run_dvc``.
"""
__version__ = "0.1.0"
