// Fused-kernel instantiations: fftsize 40, 48, without a spot PSF and with a
// PSF of the same size.
#include "wfs_launch.cuh"

SHWFS_REGISTER_PLAIN(40, 0)
SHWFS_REGISTER_PLAIN(40, 40)
SHWFS_REGISTER_PLAIN(48, 0)
SHWFS_REGISTER_PLAIN(48, 48)
