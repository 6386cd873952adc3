"""lmff_gb300: GB300 (sm_103a) engine for the Tersoff + ILP layered-materials path.

Submodules: ``capi`` (ctypes binding of include/lmff_gb300.h), ``build`` (in-tree nvcc
build of liblmff_gb300.so), ``structures`` (seeded layered-system generators),
``serve`` (continuous-batching request loop), ``tune`` (launch-shape autotuner).
"""
