// Error handling and small device-memory helpers shared by the CUDA sources.
#pragma once
#include <cuda_runtime.h>

#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/pecs.h"

namespace pecs {

struct PecsError : std::runtime_error {
  int code;
  PecsError(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

#define PECS_CUDA(x)                                                                        \
  do {                                                                                      \
    cudaError_t e_ = (x);                                                                   \
    if (e_ != cudaSuccess)                                                                  \
      throw ::pecs::PecsError(PECS_E_CUDA, std::string(#x) + ": " + cudaGetErrorString(e_)); \
  } while (0)

// Owning device buffer.
template <typename T>
struct DBuf {
  T* p = nullptr;
  size_t n = 0;
  DBuf() = default;
  DBuf(const DBuf&) = delete;
  DBuf& operator=(const DBuf&) = delete;
  DBuf(DBuf&& o) noexcept : p(o.p), n(o.n) {
    o.p = nullptr;
    o.n = 0;
  }
  DBuf& operator=(DBuf&& o) noexcept {
    if (this != &o) {
      release();
      p = o.p;
      n = o.n;
      o.p = nullptr;
      o.n = 0;
    }
    return *this;
  }
  ~DBuf() { release(); }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
  }
  void alloc(size_t count) {
    release();
    if (count == 0) return;
    PECS_CUDA(cudaMalloc(&p, count * sizeof(T)));
    n = count;
  }
  void upload(const T* h, size_t count) {
    alloc(count);
    if (count) PECS_CUDA(cudaMemcpy(p, h, count * sizeof(T), cudaMemcpyHostToDevice));
  }
  void upload(const std::vector<T>& v) { upload(v.data(), v.size()); }
  void zero() {
    if (n) PECS_CUDA(cudaMemset(p, 0, n * sizeof(T)));
  }
};

}  // namespace pecs
