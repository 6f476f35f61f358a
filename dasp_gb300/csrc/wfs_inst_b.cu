// Fused-kernel instantiations: fftsize 16, 24, without a spot PSF and with a
// PSF of the same size.
#include "wfs_launch.cuh"

SHWFS_REGISTER_PLAIN(16, 0)
SHWFS_REGISTER_PLAIN(16, 16)
SHWFS_REGISTER_PLAIN(24, 0)
SHWFS_REGISTER_PLAIN(24, 24)
