// Fused-kernel instantiations: fftsize 32, without a spot PSF and with a
// PSF of the same size.
#include "wfs_launch.cuh"

SHWFS_REGISTER_PLAIN(32, 0)
SHWFS_REGISTER_PLAIN(32, 32)
