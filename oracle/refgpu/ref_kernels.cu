// ref_kernels.cu - TEST INFRASTRUCTURE ONLY: one translation unit that compiles the reference's
// own device code (MarWo22/master_thesis src/cuda_compute/kernel_settings.cu,
// plate_tectonics_kernel.cu, ccl.cu, included where they lie by oracle/Makefile's `refgpu`
// target) into a relocatable sm_103a cubin under oracle/_ref/.  The GPU harness
// (ref_gpu_harness.cpp) links it at run time and launches the reference's kernels to time them
// beside the engine.  Nothing from the reference is copied into the repository.
#include "kernel_settings.cu"
#include "plate_tectonics_kernel.cu"
#include "ccl.cu"
