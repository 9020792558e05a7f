// ref_export.cu - TEST INFRASTRUCTURE ONLY: compiles the reference's image export
// (MarWo22/master_thesis src/cuda_compute/texture_save.cu, included where it lies by
// oracle/Makefile's `refexport` target) into an sm_103a cubin under oracle/_ref/, so that GPU
// tests can run its two conversion kernels (convertGrayscaleToRgbKernel,
// convertFloatToGray16Kernel) and compare the engine's exports with them.  stubs_png/ declares
// the libpng names the host half of that file uses; none is called.
#include "texture_save.cu"
