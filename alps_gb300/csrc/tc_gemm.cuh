// tc_gemm.cuh -- FP64-accurate dense products on the BF16 tensor cores
// (tc_gemm.cu).
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>

// slices per operand (7 x 8 bits: 55 bits of each row's / column's scale)
#define TC_SLICES 7

// Device workspace tc_product needs for an M x N x K product.
size_t tc_workspace_bytes(int M, int N, int K);

// C = beta C + alpha A B on the tensor cores (K <= 256); A (M x K) at
// A[r*ars + k*aks], B (K x N) at B[k*bks + c*bcs], C at C[r*crs + c*ccs].
// kexp (length K, device, may be null): A's column k is scaled by
// 2^kexp[k] and B's row k by 2^-kexp[k] before slicing.  bound (may be
// null): per entry the fixed-point scale 2^(eA_r + eB_c); the entry's error
// is at most 10 K 2^-56 |alpha| times it.  Asynchronous on st.
int tc_product(const double* A, long ars, long aks, const double* B, long bks, long bcs, double* C, long crs,
               long ccs, int M, int N, int K, double alpha, double beta, const int* kexp, void* ws, double* bound,
               cudaStream_t st);

// Device addresses of the row and column exponents inside ws.
void tc_exponents(const void* ws, int M, int N, int K, const int** eA, const int** eB);

// Error word of the last tc_product on ws (synchronous): ALPS_OK or
// ALPS_E_TIMEOUT when a bounded wait of the kernel ran out.
int tc_check(const void* ws, int M, int N, int K);

// C = A B (A M x K row-major, B K x N row-major, C M x N row-major, K <= 256)
// with FP64 accuracy per entry: the product runs on the tensor cores after
// scaling B's rows (and A's columns) by powers of two to unit size, and
// every entry whose fixed-point error bound exceeds 2^-44 sum_k |A_rk B_kc|
// (the size of FP64 GEMM's own worst-case rounding bound) is recomputed in
// FP64.  *fixed (may be null, host) receives the number of such entries
// after a synchronisation.  ws: tc_checked_workspace_bytes(M, N, K).
size_t tc_checked_workspace_bytes(int M, int N, int K);
int tc_product_checked(const double* A, const double* B, double* C, int M, int N, int K, void* ws, int* fixed,
                       cudaStream_t st);
