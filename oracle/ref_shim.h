/*
 * Force-included (nvcc -include) when the reference's device code is compiled
 * into cubins by oracle/build_ref.py. Test infrastructure only.
 *
 * The reference's QR/panel.cu includes its vendored CUB 1.8.0
 * (include/cub-1.8.0), whose tex_ref_input_iterator.cuh names the texture
 * reference template that CUDA 12 removed. No reference kernel on the QR path
 * uses that iterator; declaring an empty template of that name lets the file
 * compile unchanged. (The other two compile flags the recipe adds:
 * CUB_NS_QUALIFIER, which CUDA 13's own CUB requires once the vendored copy
 * has defined CUB_NS_PREFIX, and a macro standing in for
 * cudaDeviceProp::clockRate, removed in CUDA 13, in util/util.cu's host-only
 * print_env.)
 */
#pragma once
template <typename T>
struct texture {
  int normalized;
};
