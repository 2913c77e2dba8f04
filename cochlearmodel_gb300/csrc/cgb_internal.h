// Internal helpers shared by the translation units of libcochlea_gb300.so.
#pragma once

#include <cstdint>
#include <string>

#include "cochlea_gb300.h"

namespace cgb {

// Records msg as the last error of the calling thread and returns code.
int fail(int code, const std::string& msg);
// Checks a CUDA runtime status; on failure records "<what>: <cuda message>".
int cuda_check(int cuda_status, const char* what);
void note_launch();
// A host mirror receives a kernel's results by device stores over the
// CPU-GPU link: it must be pinned host memory mapped into the device address
// space at the same address (cudaHostAlloc, or cudaHostRegister with the
// mapped flag, under unified addressing) and 16-byte aligned.
int check_host_mirror(const void* p, const char* what);

}  // namespace cgb

#define CGB_TRY_CUDA(call, what)                               \
  do {                                                         \
    int _st = (int)(call);                                     \
    if (_st != 0) return ::cgb::cuda_check(_st, what);         \
  } while (0)
