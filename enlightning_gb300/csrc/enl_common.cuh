// Shared definitions of the enlightning_gb300 CUDA library.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/enlightning_gpu.h"

namespace enl {

// Library-wide state (enl_common.cu).
cudaStream_t stream();
void set_error(int code);
int check_launch(const char* where);
int* device_health_word();

constexpr int kNequ = 5;
constexpr int kGhost = 3;
constexpr int kReflect = 10;
constexpr int kAbsorb = 20;

// Strided view of a block of fields: field k, canvas cell (i, j) lives at
// base[k * fstride + j * pitch + i], where (i, j) = (0, 0) is the first
// stored cell (the lower-left ghost cell for a ghosted SAMRAI array).
template <typename T>
struct Fields {
  T* base;
  long pitch;
  long fstride;
  __host__ __device__ T& at(int k, int i, int j) const {
    return base[(long)k * fstride + (long)j * pitch + i];
  }
};

// Reference REAL*4 literals widened to double (rhs_hybrid_high_llf.m4 and
// siblings, tag_cells.m4): the value of the single-precision constant.
struct Lit {
  static constexpr double c0_9 = (double)0.9f;
  static constexpr double c0_9999 = (double)0.9999f;
  static constexpr double c0_78 = (double)0.78f;
  static constexpr double c4_3 = (double)(4.0f / 3.0f);
  static constexpr double c2_3 = (double)(2.0f / 3.0f);
  static constexpr double c1_3 = (double)(1.0f / 3.0f);
  static constexpr double c13_12 = (double)(13.0f / 12.0f);
  static constexpr double c1_6 = (double)(1.0f / 6.0f);
  static constexpr double c0_1 = (double)0.1f;
  static constexpr double c0_6 = (double)0.6f;
  static constexpr double c0_3 = (double)0.3f;
  static constexpr double weno_eps = (double)10.0e-6f;
  static constexpr double a1 = (double)0.79926643f;
  static constexpr double a2 = (double)-0.18941314f;
  static constexpr double a3 = (double)0.02651995f;
};

}  // namespace enl
