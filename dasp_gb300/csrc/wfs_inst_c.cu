// Fused-kernel instantiations: fftsize 20, without a spot PSF and with a
// PSF of the same size.
#include "wfs_launch.cuh"

SHWFS_REGISTER_PLAIN(20, 0)
SHWFS_REGISTER_PLAIN(20, 20)
