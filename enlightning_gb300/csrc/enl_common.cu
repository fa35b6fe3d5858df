// Library-wide state: stream, sticky error word, scheme selection.
#include <cstdio>
#include <cstdlib>

#include "enl_common.cuh"

namespace enl {

static cudaStream_t g_stream = nullptr;
static int g_last_error = ENL_OK;
static int g_rhs_variant = ENL_HYBRID_HIGH_LLF;

cudaStream_t stream() { return g_stream; }

void set_error(int code) {
  if (g_last_error == ENL_OK) g_last_error = code;
}

static int sync_check() {
  static int v = -1;
  if (v < 0) {
    const char* s = getenv("ENL_SYNC_CHECK");
    v = (s && s[0] == '1') ? 1 : 0;
  }
  return v;
}

int check_launch(const char* where) {
  if (sync_check()) {
    cudaError_t se = cudaDeviceSynchronize();
    if (se != cudaSuccess) fprintf(stderr, "enlightning_gpu: %s (sync): %s\n", where, cudaGetErrorString(se));
  }
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    fprintf(stderr, "enlightning_gpu: %s: %s\n", where, cudaGetErrorString(e));
    set_error(ENL_ERR_CUDA);
    return ENL_ERR_CUDA;
  }
  return ENL_OK;
}

int rhs_variant() { return g_rhs_variant; }

}  // namespace enl

extern "C" {

int enl_set_stream(void* s) {
  enl::g_stream = (cudaStream_t)s;
  return ENL_OK;
}

int enl_get_last_error(void) {
  int e = enl::g_last_error;
  enl::g_last_error = ENL_OK;
  return e;
}

const char* enl_error_string(int code) {
  switch (code) {
    case ENL_OK: return "ok";
    case ENL_ERR_ARG: return "invalid argument";
    case ENL_ERR_CUDA: return "CUDA error";
    case ENL_ERR_NONFINITE: return "non-finite or non-positive density in the state";
    case ENL_ERR_TIMEOUT: return "bounded device wait expired";
    case ENL_ERR_STATE: return "invalid call order";
    default: return "unknown error";
  }
}

int enl_set_rhs_variant(int v) {
  if (v < 0 || v > 8) {
    enl::set_error(ENL_ERR_ARG);
    return ENL_ERR_ARG;
  }
  enl::g_rhs_variant = v;
  return ENL_OK;
}

int enl_get_rhs_variant(void) { return enl::g_rhs_variant; }

}  // extern "C"
