// hs_noalloc.h -- fixed-storage inject writes (see hs_noalloc.cu).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <mutex>

namespace hsg {

// One write: *addr = value and, when flag is not null, *flag = 1.
struct InjectWrite {
    double* addr;
    uint8_t* flag;
    double value;
};

// Most writes per call (the size of the host staging and device scratch).
constexpr uint32_t kInjectWriteMax = 32768;

std::mutex& injectStaticLock();
InjectWrite* injectStaging();
cudaError_t scatterInjectStatic(int device, uint32_t n, cudaStream_t st);

}  // namespace hsg
