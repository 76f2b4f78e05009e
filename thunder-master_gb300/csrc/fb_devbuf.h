// fb_devbuf.h -- growable device buffer of libfbgpu (host side).
#pragma once
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cstddef>

#include "../../include/fbgpu.h"

namespace fb {

// bumped by every device (re)allocation: a captured CUDA graph whose
// pointers may have moved is re-captured
extern std::atomic<long long> g_alloc_gen;

// device buffer that grows on demand and never shrinks
struct DevBuf {
  void *p = nullptr;
  size_t cap = 0;
  int ensure(size_t bytes) {
    if (bytes <= cap) return 0;
    if (p) cudaFree(p);
    p = nullptr;
    cap = 0;
    size_t want = std::max<size_t>(bytes, 256);
    if (cudaMalloc(&p, want) != cudaSuccess) return FB_ERR_CUDA;
    cap = want;
    g_alloc_gen++;
    return 0;
  }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    cap = 0;
  }
  template <class T>
  T *as() const {
    return static_cast<T *>(p);
  }
};

}  // namespace fb
