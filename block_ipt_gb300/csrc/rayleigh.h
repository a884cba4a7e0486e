// rayleigh.h - pieces of the Rayleigh-mixed drivers (abi_rayleigh.cu), shared
// with the Rayleigh ACX entry (k_acx.cu).  Internal.
#pragma once

#include <cuda_runtime.h>

#include "block_ops.h"

namespace iptgb {

// Q = the orthonormal basis of X0 (n x k, column-major) with the column
// signs of LAPACK's Householder QR (CholQR2 in FP64, signs from the top
// k x k block); X0 is overwritten.  Invalid argument when the block is
// numerically rank deficient.
int householder_basis(BlockOps &ops, double *X0, int n, int k, double *Q, cudaStream_t s);

// B = sym(Q^T H Q) in FP64 (k x k), H column-major n x n.
int projected_matrix(BlockOps &ops, const double *dH, int n, const double *Q, int k, double *B,
                     cudaStream_t s);

}  // namespace iptgb
