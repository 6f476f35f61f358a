"""GB300-native Shack-Hartmann wavefront-sensor engine.

A drop-in for the per-frame WFS step of the Durham AO Simulation Platform
(``util.centcmod`` over ``cmod.cent``): phase -> spot images -> centroids in
hand-written sm_103a CUDA behind a C ABI (``include/shwfs.h``).

Use it as the reference module is used::

    import dasp_gb300.centcmod
    c = dasp_gb300.centcmod.centcmod(nthreads, nsubx, ...)
"""
