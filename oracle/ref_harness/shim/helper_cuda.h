/* stand-in for the CUDA samples helper: error checking only */
#pragma once
#include <cstdio>
#include <cstdlib>
template <typename T>
inline void gv_check_cuda(T result, const char* what) {
  if (result) { std::fprintf(stderr, "CUDA error %d at %s\n", (int)result, what); std::exit(1); }
}
#define checkCudaErrors(val) gv_check_cuda((val), #val)
