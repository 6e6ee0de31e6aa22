// Shared pieces of the Nektar++ adapter classes that put the GB300 library behind the
// reference's Collections::Operator and GlobalLinSys factories (see CollectionsGPU.cpp,
// GlobalLinSysGPU.cpp). These files are meant to be added to a Nektar++ build (library/
// Collections and library/MultiRegions) and linked with -lithaca_gpu; the repository
// compiles and links them against stand-in headers of the same signatures.
#pragma once

#include <map>
#include <mutex>

#include <ithaca_gpu.h>

namespace Nektar {
namespace GpuAdapter {

// One process-wide library context on device 0, created on first use.
inline ithaca_gpu_ctx* GpuContext() {
  static ithaca_gpu_ctx* ctx = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    if (ithaca_gpu_ctx_create(0, &ctx) != ITHACA_GPU_OK) ctx = nullptr;
  });
  return ctx;
}

// A non-zero status of the C ABI becomes the reference's NekError.
inline void Check(int rc) {
  if (rc != ITHACA_GPU_OK) {
    char msg[512];
    ithaca_gpu_last_error(msg, sizeof msg);
    throw ErrorUtil::NekError(std::string("ithaca_gpu: ") + msg);
  }
}

// The FP64 collection operator of a set of elements, keyed by its first element
// expansion: the Collections operators register theirs, and a global system built on the
// same expansion list (ExpList::GetExp(0)) finds it.
inline std::map<const void*, ithaca_gpu_op*>& OperatorRegistry() {
  static std::map<const void*, ithaca_gpu_op*> r;
  return r;
}

}  // namespace GpuAdapter
}  // namespace Nektar
