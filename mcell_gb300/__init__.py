"""mcell_gb300: GB300 (sm_103a) engine for MCell4's volume-molecule diffuse-react step.

The compute path is CUDA behind a C ABI (include/mcell_gb300.h); Python calls it
through ctypes (mcell_gb300._native). mcell_gb300.workloads builds the synthetic
models of the benchmark configurations; mcell_gb300.conversion restates the
Model API's unit conversions (space steps, reaction probabilities, partitions).
"""
__version__ = "0.1.0"
