// Run-time compiled network kernels (ssa_jit.cpp).
#pragma once

#include <cuda_runtime.h>

#include <string>

#include "network.hpp"
#include "ssa_args.hpp"

namespace rbg {

// Networks the generator covers: 1..16 species, 1..32 reactions, jumps of
// magnitude below 2^23.
bool jit_supported(const Packed &p);
// CUDA source of the speculative kernel specialised for the network, for
// blocks of `block` lanes (a multiple of 32, at most 1024).
std::string jit_net_source(const Packed &p, int block);
// Compile (or find in the disk cache) the network's kernel image without
// loading it; false with the error set on failure.
bool jit_compile(const Packed &p, int block, size_t *image_bytes);
// The compiled kernel for the current device (compiled on first use); null
// with the error set on failure.  With `compile` false only a kernel already
// loaded or in the disk cache is returned (null, no error, otherwise).  A
// kernel built for `block` lanes also runs blocks of fewer lanes.
const void *jit_kernel(const Packed &p, int block, bool compile = true);
// Compile the network's kernel into the disk cache on a background thread
// (once per generated source), so that a later run finds it there.
void jit_compile_async(const Packed &p, int block);
int launch_ssa_jit(const void *kern, const SsaArgs &a, int block, int grid, size_t smem, cudaStream_t st);
// Lanes per block of a generated kernel for a full-size ensemble: 384 (12
// warps per SM at up to 168 registers a lane; fastest measured on the dimer and
// Vilar networks), or RB_JIT_BLOCK rounded to a multiple of 32.
int jit_block();

}  // namespace rbg
