// sg_setup.h -- graph setup on the GPU (see sg_setup.cu).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

// CSR on the device from an edge list in agent ids. ids[0..n): the agents' ids in
// buffer order (distinct, not INT64_MIN); edges (src[k], dst[k]), k < m, host
// arrays. undirected adds every edge in both directions; ordered keeps each row in
// first-connection order (else rows are sorted by neighbour index); repeated
// edges are dropped. On SG_OK *d_off (n + 1) and *d_idx (*nnz_out, at least one
// slot) are cudaMalloc'ed device arrays the caller owns. On failure *why says why.
int sg_build_csr_from_ids(const int64_t *ids, int64_t n, const int64_t *src, const int64_t *dst, int64_t m,
                          bool undirected, bool ordered, cudaStream_t st, int32_t **d_off, int32_t **d_idx,
                          int64_t *nnz_out, std::string *why);
