// Fused-kernel instantiations: fftsize 25, 30, without a spot PSF and with a
// PSF of the same size.
#include "wfs_launch.cuh"

SHWFS_REGISTER_PLAIN(25, 0)
SHWFS_REGISTER_PLAIN(25, 25)
SHWFS_REGISTER_PLAIN(30, 0)
SHWFS_REGISTER_PLAIN(30, 30)
