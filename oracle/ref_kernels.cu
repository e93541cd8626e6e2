// Translation unit that makes nvcc emit the reference's own SDGC kernels
// (bf_inference, snig_inference, identify) from their headers in the
// reference tree; built by oracle/ref_build.sh into oracle/_ref/ (never
// committed) and loaded by oracle/ref_harness.cpp on a GPU.  Test
// infrastructure only.
#include <cstddef>
#include <thrust/reduce.h>   // utility.hpp:203 uses thrust::reduce without including it
#include <utility.hpp>
#include <BF/kernel.hpp>
#include <SNIG/kernel.hpp>
