"""mcell_gb300: GB300 (sm_103a) engine for MCell4's volume-molecule diffuse-react step.

The compute path is CUDA behind a C ABI (include/mcell_gb300.h); Python calls it
through ctypes (mcell_gb300._native). mcell_gb300.model mirrors the parts of the
pymcell4 Model API that describe a volume-reaction model.
"""
__version__ = "0.1.0"
