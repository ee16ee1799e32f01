// sg_step_rt.h -- NVRTC compilation and launch of user step functions.
//
// Replaces SAGESim's codegen + CuPy-JIT pipeline (sagesim/model.py:800-865
// writes and imports a generated module; model.py:2010-2457 builds the fused
// kernel around the AST-rewritten step functions). Here the user step is CUDA
// C++ against the sg_ctx API of include/sagesim_gb300_step.h; the engine wraps
// it in a tile-walking kernel, compiles it for the device's architecture with
// NVRTC (loaded with dlopen on first use, so the library itself has no NVRTC
// link dependency) and loads the cubin with cudaLibraryLoadData.
#pragma once
#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "../../include/sagesim_gb300_step.h"

struct SgCompiledStep;

// Compiles `src` (defining `entry`) into a kernel for `device`.
// Returns SG_OK, SG_ERR_COMPILE (log holds the NVRTC log) or SG_ERR_CUDA.
int sg_step_rt_compile(int device, const char *src, const char *entry, SgCompiledStep **out,
                       std::string *log);
cudaError_t sg_step_rt_launch(SgCompiledStep *s, const sg_step_args &a, int grid, cudaStream_t st);
void sg_step_rt_destroy(SgCompiledStep *s);
// The source the engine hands NVRTC for a given step (for tests and docs).
std::string sg_step_rt_source(const char *src, const char *entry);
