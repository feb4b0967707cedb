"""GB300-native (sm_103a) simulation hot path of patchV1 (zhaobenyan51129/visual-cortex).

The LGN convolution and Poisson spikes, the conductance-based LIF/AdEx step and the near and
far spike delivery run as hand-written CUDA kernels behind the C ABI of
include/patchv1_gb300.h; this package is the host side (cfg parsing, file formats, driver).
"""
__version__ = "0.1.0"
