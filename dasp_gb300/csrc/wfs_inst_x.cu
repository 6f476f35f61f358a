// Fused-kernel instantiations whose spot PSF differs in size from the FFT:
// a PSF larger than fftsize (power spectrum zero-padded, addPowerSpecCentral
// with psfsize > fftsize) and pre-binning (preBinningFactor 2: paddedsize =
// fftsize, PSF of fftsize/2).
#include "wfs_launch.cuh"

SHWFS_REGISTER_PLAIN(16, 32)
SHWFS_REGISTER_PLAIN(20, 40)
SHWFS_REGISTER_PLAIN(32, 16)
SHWFS_REGISTER_PLAIN(40, 20)
SHWFS_REGISTER_PLAIN(64, 32)
