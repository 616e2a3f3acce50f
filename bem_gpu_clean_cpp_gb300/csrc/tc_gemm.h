// FP32-accurate real GEMMs on the tcgen05 tensor cores (fp16 split
// products, FP32 accumulation in tensor memory), used for the dense
// contractions of the solve: the multi-right-hand-side products A X and
// A^H T of block GMRES and the trailing updates of the blocked Householder
// QR.  See tc_gemm.cu for the method and its accuracy.
#pragma once

#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <cstddef>

namespace bem {

constexpr int kTcKP = 64;        // K padding of a packed right-hand operand (one stage)
constexpr int kTcColPad = 256;   // column padding of a packed right-hand operand

// The right-hand operand B (K x ncols real) packed for tc_gemm: P fp16
// planes (hi, lo or hi, mid, lo) of B's columns scaled by a power of two per
// column, plane p at planes + p * ncols_pad * Kp, column n of a plane as Kp
// contiguous halfs (zero beyond K); col_inv[n] = 1 / column n's scale.
struct TcOperand {
    __half *planes = nullptr;
    float *col_inv = nullptr;
    int K = 0, Kp = 0, ncols = 0, ncols_pad = 0, P = 2;
};

// Device bytes of a packed operand (planes + scales).
size_t tc_operand_bytes(int K, int ncols, int P);
// Lays out a packed operand in `mem` (tc_operand_bytes(K, ncols, P) bytes).
TcOperand tc_operand_view(void *mem, int K, int ncols, int P);

// Packs a real matrix (K x ncols, column-major, leading dimension ld) into op.
void tc_pack_real(const float *B, size_t ld, TcOperand &op, cudaStream_t st);
// Packs the complex block X (n x S, column-major, leading dimension ldx, n
// when 0) as the interleaved real right-hand block (2n x 2S): column s holds
// (Re x_j, -Im x_j) at rows (2j, 2j+1) and column S + s holds (Im x_j, Re
// x_j), so that the interleaved real view of a complex matrix L (rows of
// (re, im) pairs) times it gives Re(L x) in column s and Im(L x) in column S
// + s.  conj_left: the block for conj(L) x instead ((Re x_j, Im x_j) and
// (Im x_j, -Re x_j)).
void tc_pack_cplx_f32(const float2 *X, int n, int S, TcOperand &op, cudaStream_t st, size_t ldx = 0,
                      bool conj_left = false);
void tc_pack_cplx_f64(const double2 *X, int n, int S, TcOperand &op, cudaStream_t st, size_t ldx = 0,
                      bool conj_left = false);

// scale[0] = a power of two that brings max |A| into [2^14, 2^15), scale[1]
// = its inverse, for the rows x cols real matrix A (row stride ld floats).
void tc_a_scale(const float *A, size_t ld, int rows, int cols, float *scale, cudaStream_t st);

// C (M x ncols, column-major, leading dimension ldc) = op(A) B, where A is a
// real FP32 matrix with row stride lda (floats; a multiple of 4) read
// directly from global memory: trans = false: op(A) = A (M x K); trans =
// true: op(A) = A^T with A stored K x M.  a_scale: tc_a_scale's pair (device).
// B: a packed operand (B.K == K).  part: scratch of part_floats floats for
// split-K partial sums, at least tc_gemm_part_floats() of this shape (may be
// null when that is 0; a plan that needs more is refused).  status:
// device word set to 1 if a bounded wait of the kernel timed out (the result
// is then invalid).  Deterministic: the same inputs give the same bits.
// subtract: C -= op(A) B instead of C = op(A) B.
void tc_gemm(const float *A, size_t lda, bool trans, int M, int K, const float *a_scale, const TcOperand &B,
             float *C, size_t ldc, float *part, size_t part_floats, int *status, cudaStream_t st,
             bool subtract = false);
size_t tc_gemm_part_floats(int M, int K, int ncols, int P);
// Upper bound of tc_gemm_part_floats over K, P and the device's SM count.
size_t tc_gemm_part_floats_bound(int M, int ncols);

}  // namespace bem
