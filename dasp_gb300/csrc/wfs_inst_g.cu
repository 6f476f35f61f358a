// Fused-kernel instantiations: fftsize 50, 60, without a spot PSF and with a
// PSF of the same size.
#include "wfs_launch.cuh"

SHWFS_REGISTER_PLAIN(50, 0)
SHWFS_REGISTER_PLAIN(50, 50)
SHWFS_REGISTER_PLAIN(60, 0)
SHWFS_REGISTER_PLAIN(60, 60)
