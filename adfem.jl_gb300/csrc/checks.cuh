// Index checks of the debug build (compiled with -DADFEM_CHECKS; release builds compile them
// out).  A kernel checks an index it computed before it uses it; a failing check records the
// source line in this translation unit's flag (the first failure wins) and the caller
// redirects the access to an index that is known to be valid, so the kernel finishes and the
// host learns of it through adfem_debug_check_code().  Nothing traps.
#pragma once
#include <cuda_runtime.h>

#ifdef ADFEM_CHECKS
static __device__ int g_check_line;
__device__ __forceinline__ bool adfem_check(bool ok, int line) {
  if (!ok) atomicCAS(&g_check_line, 0, line);
  return ok;
}
#define ADFEM_DCHECK(cond) adfem_check((cond), __LINE__)
// host: the recorded line (0: none), cleared; -1 if the flag cannot be read
#define ADFEM_CHECK_READER(name)                                                   \
  int name() {                                                                     \
    int v = 0, z = 0;                                                              \
    if (cudaMemcpyFromSymbol(&v, g_check_line, sizeof(int)) != cudaSuccess) return -1; \
    cudaMemcpyToSymbol(g_check_line, &z, sizeof(int));                             \
    return v;                                                                      \
  }
#else
#define ADFEM_DCHECK(cond) true
#define ADFEM_CHECK_READER(name) \
  int name() { return 0; }
#endif
