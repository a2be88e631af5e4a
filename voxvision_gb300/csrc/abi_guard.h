/*
 * abi_guard.h -- no C++ exception crosses the library's C ABI.
 *
 * An exported function written in C++ is a function-try-block:
 *
 *     EXPORT int vox_cuda_x(...)
 *     try {
 *         ...
 *     } VOX_ABI_FAIL_INT
 *
 * and its handler returns the call's failure value.  All the library's own
 * code can throw is an allocation or thread-creation failure (std::bad_alloc,
 * std::system_error from the standard containers, mutexes and threads), so
 * the status calls report VOX_CUDA_ENOMEM.
 */
#ifndef VOX_ABI_GUARD_H
#define VOX_ABI_GUARD_H

#include "../../include/voxtrees_cuda.h"

#define VOX_ABI_FAIL_INT  catch (...) { return VOX_CUDA_ENOMEM; }
#define VOX_ABI_FAIL_NULL catch (...) { return nullptr; }
#define VOX_ABI_FAIL_ZERO catch (...) { return 0; }
#define VOX_ABI_FAIL_VOID catch (...) { return; }

#endif
