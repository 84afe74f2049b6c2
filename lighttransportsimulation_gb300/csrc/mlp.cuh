// Radiance-cache MLP on the 5th-generation tensor cores (host interface of mlp.cu).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

namespace lts {

// Tensor-core product check: D = op(A) op(B) for the three operand arrangements the MLP uses
// (mode 0: K-major x K-major, 128x64 . (64x64)^T; mode 1: K-major x MN-major, 128x64 . 64x96;
// mode 2: MN-major x MN-major, (128x96)^T . 128x64 with M padded to 128).  Host buffers of bf16
// bits; D is 128 x 64 or 128 x 96 FP32.  swap exchanges the two byte offsets of MN-major
// descriptors (a layout check).
std::string umma_probe(int mode, int swap, const uint16_t* a, const uint16_t* b, float* d, uint32_t* d_err,
                       cudaStream_t s);

}  // namespace lts
