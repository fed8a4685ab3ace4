// Dense FP64 complex helpers for the GCG eigensolver (see k_dense.cu).
#pragma once
#include <cuda_runtime.h>

#include <cstddef>

namespace ncgm {

// C (p x q, ld ldc) = A^H B; partials: >= maxChunks * p * q double2.
void gram(const double2 *A, size_t lda, int p, const double2 *B, size_t ldb,
          int q, size_t N, double2 *C, int ldc, double2 *partials,
          int maxChunks, cudaStream_t s);
int gramMaxChunks();
// C = A^H B on the tensor cores (tcgen05 kind::tf32, split TF32 products,
// FP32 accumulation over row chunks, FP64 chunk sums; k_tcgram.cu). part:
// tcGramPartialFloats(N, p, q) floats.
void gramTC(const double2 *A, size_t lda, int p, const double2 *B, size_t ldb,
            int q, size_t N, double2 *C, int ldc, float *part,
            cudaStream_t s);
size_t tcGramPartialFloats(size_t N, int p, int q);
int *tcGramErrWord();
// C = A^H B on the tensor cores to ~1e-13 relative: error-free splitting into
// BF16 integer digits (digitised once per operand), exact FP32 level sums,
// exact 64-bit combination (k_tcgram_exact.cu). scratch:
// exactGramScratchDoubles(N, p, q) doubles, 16-byte aligned.
void gramTCExact(const double2 *A, size_t lda, int p, const double2 *B,
                 size_t ldb, int q, size_t N, double2 *C, int ldc,
                 double *scratch, cudaStream_t s);
size_t exactGramScratchDoubles(size_t N, int p, int q);
int *exactGramErrWord();
// Y = V C on the tensor cores with the exact digit products of gramTCExact
// (~1e-12 relative of the column maxima; k_tcgram_exact.cu). scratch:
// exactVCScratchBytes(N, m, k) bytes, 16-byte aligned.
void gemmVCExact(const double2 *V, size_t ldv, int m, const double2 *C,
                 int ldc, int k, double2 *Y, size_t ldy, size_t N,
                 void *scratch, cudaStream_t s, bool accum = false);
size_t exactVCScratchBytes(size_t N, int m, int k);
// Y = V C + beta Y (V: N x m with m <= 1600, C: m x k; C is staged in
// shared memory in blocks of columns).
void gemmVC(const double2 *V, size_t ldv, int m, const double2 *C, int ldc,
            int k, double2 *Y, size_t ldy, size_t N, double beta,
            cudaStream_t s);
// Cholesky of Gram G with MGS-equivalent drop; T = R^{-1}; keep flags.
// fast: the FP32 forms' variant (double-float pivot roots and reciprocals).
void cholDrop(const double2 *G, int ldg, int m, double dropTol, double2 *R,
              double2 *T, int *keep, cudaStream_t s, bool fast = false);
// Multi-kernel Hermitian eigensolver for m > 80 (k_heig_large.cu): Householder
// tridiagonalisation, bisection, inverse iteration, back-transformation.
void heigLarge(const double2 *A, int lda, int m, double2 *V, double *w,
               int *perm, int *status, void *scratch, cudaStream_t s);
size_t heigLargeScratchBytes(int m);
// The same method with the tridiagonalisation in one CTA and the matrix in
// shared memory, for m <= heigMidMax() (k_heig_large.cu).
void heigMid(const double2 *A, int lda, int m, double2 *V, double *w,
             int *perm, int *status, void *scratch, cudaStream_t s);
size_t heigMidScratchBytes(int m);
int heigMidMax();
// Hermitian eigensolver (lower triangle): w ascending, V eigenvectors (m x m).
// fast (the FP32 precision forms): for m <= heigMidMax(), the one-CTA
// double-float Householder method (heigMid; with NCGM_HEIG_MID=0 the
// double-float Jacobi up to m = 80); otherwise the FP64 Jacobi up to m = 80
// and the multi-kernel Householder method above it. Degenerate eigenvectors
// may come out rotated within their eigenspace between the methods.
// scratch (optional, heigScratchBytes(m) bytes): the Householder methods'
// workspace; without it they take stream-ordered allocations per call.
void heig(const double2 *A, int lda, int m, double2 *work, double2 *V,
          double *w, int *perm, int *status, cudaStream_t s,
          bool fast = false, void *scratch = nullptr,
          size_t scratchBytes = 0);
size_t heigScratchBytes(int m);

} // namespace ncgm
