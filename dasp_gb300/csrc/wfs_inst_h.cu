// Fused-kernel instantiations: fftsize 64, without a spot PSF and with a
// PSF of the same size.
#include "wfs_launch.cuh"

SHWFS_REGISTER_PLAIN(64, 0)
SHWFS_REGISTER_PLAIN(64, 64)
