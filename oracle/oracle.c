/*
 * CPU oracle for the sparse hot path: a plain-C restatement of the reference's algorithms.
 *
 * TEST INFRASTRUCTURE. Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline
 * leg (and its reference arm) may load this library, and only as the checker or as the
 * timed CPU baseline. The product path (armsparse_gb300) never calls it.
 *
 * Pinning: tests/test_oracle_pins.py checks every function here that restates a reference
 * kernel against the reference's own code compiled from its sources by oracle/Makefile
 * (target `ref`, x86 build through a scalar NEON shim) and against the committed golden
 * vectors in tests/golden/ that tests/golden/make_golden.py produced from that build.
 *
 * Floating-point rules: this file is compiled with -ffp-contract=off, so every fused
 * multiply-add below is an explicit fmaf()/fma() and every other expression rounds after
 * each operation.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* ----------------------------------------------------------------------------------------
 * SpMM, C (+)= A*B with A in CSR and B, C dense row-major.
 * Restates rowBaseSpmm3 (SDMM.cpp:90-114) with num_vector_neon (SDMM.cpp:449-469): for
 * each row m and each stored entry idx of that row in CSR order, C[m,:] = fma(B[k,:],
 * val[idx], C[m,:]). Every output element is therefore one fused-FMA chain over the row's
 * entries in CSR order, starting from C's initial value (0 when accumulate == 0, which is
 * what a caller that zeroes C gets from the reference). The reference's scalar tail
 * (SDMM.cpp:465-467, C[i] = C[i] + A[i]*b) is fused by the compiler when FMA is available
 * (-ffp-contract=fast on AArch64), so it is a fused step here too.
 * ------------------------------------------------------------------------------------- */
void or_spmm_fma_chain_f32(int M, int N, const int *rowptr, const int *colind,
                           const float *val, const float *B, long ldb, float *C, long ldc,
                           int accumulate, int threads) {
#pragma omp parallel for num_threads(threads) schedule(static)
    for (int m = 0; m < M; ++m) {
        float *c = C + (long)m * ldc;
        if (!accumulate)
            for (int j = 0; j < N; ++j) c[j] = 0.0f;
        for (int idx = rowptr[m]; idx < rowptr[m + 1]; ++idx) {
            const float v = val[idx];
            const float *b = B + (long)colind[idx] * ldb;
            for (int j = 0; j < N; ++j) c[j] = fmaf(b[j], v, c[j]);
        }
    }
}

/* The entry-balanced GPU SpMM's summation order, restated (no reference counterpart: the
 * reference's SpMM is the single chain of or_spmm_fma_chain_f32; this states how the GPU's
 * entry-balanced kernels, spmm_nnz.cu, reorder it, so their results can be checked bit for bit).
 * The entries are cut into chunks of CH. Per output element (r, j):
 *  - each chunk's segment of row r is summed by S sub-chains: sub-chain s takes the segment's
 *    entries s, s + S, s + 2S, ... in order, fmaf from 0; the S sums are added by a butterfly
 *    (pairs s, s ^ 1, then s, s ^ 2, ...). S = 1 for the one-entry-per-step kernels (nnzsplit,
 *    whose segment sum is then the plain chain), 32 / group for the multi-entry ones (nnzme).
 *    For S = 1 a row inside one chunk starts its chain from beta * C instead of 0; for S > 1
 *    it gets fmaf(beta, C, sum) (beta != 0) at the end;
 *  - a row over n > 1 chunks: its chunk partials p_0 .. p_{n-1}, n <= 8: p_0 + p_1 + ... in
 *    order; n > 8: R consecutive runs (R = 256 / G, G = the 256-wide block of column groups of
 *    VW columns holding j: VW = 4 when N % 4 == 0, else 1), each summed from 0 in order, then
 *    run 0 + run 1 + ...; then fmaf(beta, C, t) when beta != 0. */
static float or_seg_sum(const int *colind, const float *val, const float *B, long ldb, int lo,
                        int hi, int j, int S, float init) {
    float sub[32];
    for (int s = 0; s < S; ++s) sub[s] = 0.0f;
    if (S == 1) sub[0] = init;
    for (int e = lo; e < hi; ++e) {
        const int s = (e - lo) % S;
        sub[s] = fmaf(B[(long)colind[e] * ldb + j], val[e], sub[s]);
    }
    for (int off = 1; off < S; off <<= 1) {
        float nxt[32];
        for (int s = 0; s < S; ++s) nxt[s] = sub[s] + sub[s ^ off];
        for (int s = 0; s < S; ++s) sub[s] = nxt[s];
    }
    return sub[0];
}

void or_spmm_nnz_order_f32(int M, int N, const int *rowptr, const int *colind, const float *val,
                           const float *B, long ldb, float *C, long ldc, float beta, int CH,
                           int S, int threads) {
    const int VW = N % 4 == 0 ? 4 : 1;
    const int ncg = N / VW;
#pragma omp parallel for num_threads(threads) schedule(dynamic, 16)
    for (int r = 0; r < M; ++r) {
        const int rs = rowptr[r], re = rowptr[r + 1];
        float *c = C + (long)r * ldc;
        if (rs == re) {
            for (int j = 0; j < N; ++j) c[j] = beta == 0.0f ? 0.0f : beta * c[j];
            continue;
        }
        const long c_first = rs / CH, c_last = (re - 1) / CH;
        const long n = c_last - c_first + 1;
        for (int j = 0; j < N; ++j) {
            if (n == 1) {
                if (S == 1) {
                    c[j] = or_seg_sum(colind, val, B, ldb, rs, re, j, 1,
                                      beta != 0.0f ? beta * c[j] : 0.0f);
                } else {
                    const float t = or_seg_sum(colind, val, B, ldb, rs, re, j, S, 0.0f);
                    c[j] = beta != 0.0f ? fmaf(beta, c[j], t) : t;
                }
                continue;
            }
            float t;
            if (n <= 8) {
                t = 0.0f;
                for (long q = 0; q < n; ++q) {
                    const long cc = c_first + q;
                    const int lo = (int)(cc * CH > rs ? cc * CH : rs);
                    const int hi = (int)((cc + 1) * CH < re ? (cc + 1) * CH : re);
                    const float p = or_seg_sum(colind, val, B, ldb, lo, hi, j, S, 0.0f);
                    t = q == 0 ? p : t + p;
                }
            } else {
                const int cg = j / VW, cg0 = cg / 256 * 256;
                const int cgs = ncg - cg0 < 256 ? ncg - cg0 : 256;
                const int R = 256 / cgs;
                t = 0.0f;
                for (int q = 0; q < R; ++q) {
                    const long b0 = c_first + n * q / R, b1 = c_first + n * (q + 1) / R;
                    float run = 0.0f;
                    for (long cc = b0; cc < b1; ++cc) {
                        const int lo = (int)(cc * CH > rs ? cc * CH : rs);
                        const int hi = (int)((cc + 1) * CH < re ? (cc + 1) * CH : re);
                        run += or_seg_sum(colind, val, B, ldb, lo, hi, j, S, 0.0f);
                    }
                    t = q == 0 ? run : t + run;
                }
            }
            c[j] = beta != 0.0f ? fmaf(beta, c[j], t) : t;
        }
    }
}

/* Sparse x sparse -> dense: C += A*B with A (M x K) and B (K x N) both CSR and C dense
 * row-major. For each row of A, its entries in CSR order, each contributing its B row's
 * entries in order, as the reference's sparse_matrix_mul3 does (SpMM.cpp:309-327, built with
 * FMA contraction): per output element a fused-FMA chain over A's row. */
void or_spgemm_dense_f32(int M, int N, const int *rp1, const int *ci1, const float *v1,
                         const int *rp2, const int *ci2, const float *v2, float *C, long ldc,
                         int threads) {
#pragma omp parallel for num_threads(threads) schedule(static)
    for (int m = 0; m < M; ++m) {
        float *c = C + (long)m * ldc;
        for (int idx = rp1[m]; idx < rp1[m + 1]; ++idx) {
            const int k = ci1[idx];
            const float a = v1[idx];
            for (int t = rp2[k]; t < rp2[k + 1]; ++t) c[ci2[t]] = fmaf(a, v2[t], c[ci2[t]]);
        }
    }
    (void)N;
}

/* SpMM in double precision with the per-output absolute sum sum_k |a_mk * b_kj|, used as
 * the FP64 oracle and as the scale of the relative-error metric. Inputs are double so that
 * callers can pass bf16-rounded values exactly. */
void or_spmm_f64(int M, int N, const int *rowptr, const int *colind, const double *val,
                 const double *B, long ldb, double *C, double *absC, int threads) {
#pragma omp parallel for num_threads(threads) schedule(static)
    for (int m = 0; m < M; ++m) {
        double *c = C + (long)m * N;
        double *a = absC + (long)m * N;
        for (int j = 0; j < N; ++j) { c[j] = 0.0; a[j] = 0.0; }
        for (int idx = rowptr[m]; idx < rowptr[m + 1]; ++idx) {
            const double v = val[idx];
            const double *b = B + (long)colind[idx] * ldb;
            for (int j = 0; j < N; ++j) {
                c[j] += v * b[j];
                a[j] += fabs(v * b[j]);
            }
        }
    }
}

/* ----------------------------------------------------------------------------------------
 * SpMV over the reference's 1x4-blocked "vector-aware CSR" (SpMV.cpp:15-38 builds it,
 * SpMV.cpp:155-179 consumes it): every stored block is 4 consecutive values whose first
 * column id is colInd[idx]; lane l of a 4-lane accumulator takes val[idx+l]*x[k+l]
 * (vmlaq_f32), and the row result is (s2+s0) + (s3+s1), added to y[m].
 * fused selects whether the lane update is one fused step (what GCC emits for vmlaq_f32
 * under -ffp-contract=fast) or a multiply then an add.
 * ------------------------------------------------------------------------------------- */
void or_spmv_vcsr4_f32(int M, const int *rowptr, const int *colind, const float *val,
                       const float *x, float *y, int fused, int threads) {
#pragma omp parallel for num_threads(threads) schedule(static)
    for (int m = 0; m < M; ++m) {
        float s0 = 0.f, s1 = 0.f, s2 = 0.f, s3 = 0.f;
        for (int idx = rowptr[m]; idx < rowptr[m + 1]; idx += 4) {
            const int k = colind[idx];
            if (fused) {
                s0 = fmaf(val[idx + 0], x[k + 0], s0);
                s1 = fmaf(val[idx + 1], x[k + 1], s1);
                s2 = fmaf(val[idx + 2], x[k + 2], s2);
                s3 = fmaf(val[idx + 3], x[k + 3], s3);
            } else {
                float p0 = val[idx + 0] * x[k + 0], p1 = val[idx + 1] * x[k + 1];
                float p2 = val[idx + 2] * x[k + 2], p3 = val[idx + 3] * x[k + 3];
                s0 = s0 + p0; s1 = s1 + p1; s2 = s2 + p2; s3 = s3 + p3;
            }
        }
        const float r0 = s2 + s0, r1 = s3 + s1;
        y[m] = y[m] + (r0 + r1);
    }
}

/* Build the 1x4-blocked layout from a CSR matrix with K % 4 == 0: one block per aligned
 * 4-column group that holds at least one entry, zeros filling the empty lanes, colind of
 * lane l = 4*group + l (same layout toVectorAwareCSR produces from the dense matrix,
 * SpMV.cpp:15-38). Returns the number of stored slots (4 * blocks); call with null outputs
 * to size them. */
long or_csr_to_vcsr4(int M, const int *rowptr, const int *colind, const float *val,
                     int *vrowptr, int *vcolind, float *vval) {
    long size = 0;
    for (int m = 0; m < M; ++m) {
        if (vrowptr) vrowptr[m] = (int)size;
        int idx = rowptr[m];
        while (idx < rowptr[m + 1]) {
            const int g = colind[idx] >> 2;
            if (vcolind) {
                for (int l = 0; l < 4; ++l) { vcolind[size + l] = 4 * g + l; vval[size + l] = 0.f; }
            }
            while (idx < rowptr[m + 1] && (colind[idx] >> 2) == g) {
                if (vval) vval[size + (colind[idx] & 3)] = val[idx];
                ++idx;
            }
            size += 4;
        }
    }
    if (vrowptr) vrowptr[M] = (int)size;
    return size;
}

/* y = A*x in double with the per-row absolute sum. */
void or_spmv_f64(int M, const int *rowptr, const int *colind, const double *val,
                 const double *x, double *y, double *absy) {
    for (int m = 0; m < M; ++m) {
        double s = 0.0, a = 0.0;
        for (int idx = rowptr[m]; idx < rowptr[m + 1]; ++idx) {
            s += val[idx] * x[colind[idx]];
            a += fabs(val[idx] * x[colind[idx]]);
        }
        y[m] = s;
        absy[m] = a;
    }
}

/* ----------------------------------------------------------------------------------------
 * SDDMM over a CSR pattern: out[e] = (aval ? aval[e] : 1) * <X[row(e),:], Y[col(e),:]>,
 * X is M x K and Y is N x K, both row-major (the reference's D1 and D2,
 * gcn/pytorch-custom/sddmm.cu:459-483; the reference never scales, aval == NULL
 * reproduces it). Output in CSR order.
 * or_sddmm_csr_f64: double accumulation plus the absolute sum for the error metric.
 * or_sddmm_csr_f32_lanes: the CPU baseline -- float accumulation in 8 interleaved partial
 * sums (k mod 8), combined pairwise, so that the compiler can vectorise it the way the
 * reference vectorises its own dot products (SpMV.cpp:139-154).
 * ------------------------------------------------------------------------------------- */
void or_sddmm_csr_f64(int M, int K, const int *rowptr, const int *colind, const double *aval,
                      const double *X, long ldx, const double *Y, long ldy, double *out,
                      double *absout, int threads) {
#pragma omp parallel for num_threads(threads) schedule(dynamic, 16)
    for (int m = 0; m < M; ++m) {
        const double *x = X + (long)m * ldx;
        for (int e = rowptr[m]; e < rowptr[m + 1]; ++e) {
            const double *y = Y + (long)colind[e] * ldy;
            double s = 0.0, a = 0.0;
            for (int k = 0; k < K; ++k) { s += x[k] * y[k]; a += fabs(x[k] * y[k]); }
            const double sc = aval ? aval[e] : 1.0;
            out[e] = sc * s;
            absout[e] = fabs(sc) * a;
        }
    }
}

void or_sddmm_csr_f32_lanes(int M, int K, const int *rowptr, const int *colind,
                            const float *aval, const float *X, long ldx, const float *Y,
                            long ldy, float *out, int threads) {
#pragma omp parallel for num_threads(threads) schedule(dynamic, 16)
    for (int m = 0; m < M; ++m) {
        const float *x = X + (long)m * ldx;
        for (int e = rowptr[m]; e < rowptr[m + 1]; ++e) {
            const float *y = Y + (long)colind[e] * ldy;
            float s[8] = {0, 0, 0, 0, 0, 0, 0, 0};
            int k = 0;
            for (; k + 8 <= K; k += 8)
                for (int l = 0; l < 8; ++l) s[l] = fmaf(x[k + l], y[k + l], s[l]);
            for (; k < K; ++k) s[k & 7] = fmaf(x[k], y[k], s[k & 7]);
            const float t = ((s[0] + s[4]) + (s[1] + s[5])) + ((s[2] + s[6]) + (s[3] + s[7]));
            out[e] = aval ? aval[e] * t : t;
        }
    }
}

/* Lanes per edge of the group-cooperative GPU SDDMM: about one lane per four 4-element blocks
 * of K (16 elements), a power of two up to a warp. */
static int or_sddmm_group_size(int K) {
    const int q = (K + 15) / 16;
    int g = 1;
    while (g < q && g < 32) g <<= 1;
    return g;
}

/* SDDMM in the summation order of the GPU's group-cooperative kernel: G lanes per edge
 * (or_sddmm_group_size(K)); lane l takes the 4-element blocks l, l + G, l + 2G, ... of K in
 * order with one fused-FMA chain; the lanes are then summed by a butterfly (at each step,
 * every lane adds its partner l ^ off, off = G/2 .. 1) and lane 0's value is the result.
 * Inputs are fp32 (bf16 inputs enter widened to fp32, which the GPU's bf16 kernel matches). */
void or_sddmm_csr_f32_group(int M, int K, const int *rowptr, const int *colind,
                            const float *aval, const float *X, long ldx, const float *Y,
                            long ldy, float *out, int threads) {
    const int G = or_sddmm_group_size(K);
    const int nq = (K + 3) / 4;
#pragma omp parallel for num_threads(threads) schedule(dynamic, 16)
    for (int m = 0; m < M; ++m) {
        const float *x = X + (long)m * ldx;
        for (int e = rowptr[m]; e < rowptr[m + 1]; ++e) {
            const float *y = Y + (long)colind[e] * ldy;
            float a[32], b[32];
            for (int l = 0; l < G; ++l) {
                float acc = 0.0f;
                for (int q = l; q < nq; q += G)
                    for (int i = 0; i < 4; ++i) {
                        const int k = 4 * q + i;
                        if (k < K) acc = fmaf(x[k], y[k], acc);
                    }
                a[l] = acc;
            }
            for (int off = G / 2; off >= 1; off /= 2) {
                for (int l = 0; l < G; ++l) b[l] = a[l] + a[l ^ off];
                for (int l = 0; l < G; ++l) a[l] = b[l];
            }
            out[e] = aval ? aval[e] * a[0] : a[0];
        }
    }
}

/* SDDMM in the summation order of the SpMM pass with the SDDMM fused in (the GPU's nnz-split
 * kernel, spmm_nnz.cu): out[perm ? perm[e] : e] = <X[row(e)], Y[col(e)]> where G lanes hold
 * E-element slices of K -- lane l the slices starting at (j*G + l)*E, j = 0 .. CPL-1, in that
 * order (slices at or past K skipped) -- and run one fused-FMA chain each; the lanes are then
 * summed by the butterfly of or_sddmm_csr_f32_group and lane 0's value is the result. There
 * is no reference counterpart (the reference computes no gradient for the edge values,
 * gcn/pytorch-custom/op.py:31); this states the GPU kernel's order so that its dot products
 * can be checked bit for bit. */
void or_sddmm_csr_f32_slices(int M, int K, const int *rowptr, const int *colind,
                             const float *X, long ldx, const float *Y, long ldy,
                             const int *perm, int G, int E, int CPL, float *out, int threads) {
#pragma omp parallel for num_threads(threads) schedule(dynamic, 16)
    for (int m = 0; m < M; ++m) {
        const float *x = X + (long)m * ldx;
        for (int e = rowptr[m]; e < rowptr[m + 1]; ++e) {
            const float *y = Y + (long)colind[e] * ldy;
            float a[32], b[32];
            for (int l = 0; l < G; ++l) {
                float acc = 0.0f;
                for (int j = 0; j < CPL; ++j) {
                    const int c = (j * G + l) * E;
                    if (c >= K) continue;
                    for (int i = 0; i < E; ++i) acc = fmaf(y[c + i], x[c + i], acc);
                }
                a[l] = acc;
            }
            for (int off = G / 2; off >= 1; off /= 2) {
                for (int l = 0; l < G; ++l) b[l] = a[l] + a[l ^ off];
                for (int l = 0; l < G; ++l) a[l] = b[l];
            }
            out[perm ? perm[e] : e] = a[0];
        }
    }
}

/* ----------------------------------------------------------------------------------------
 * CSR -> CSC, stable: within each column the entries keep ascending row order. This is
 * the ordering scipy's tocsc() gives on the GCN path (gcn/pytorch-custom/gcn_custom.py:52)
 * and what the reference's counting transpose (sparseTranspose.cpp:95-142: column counts,
 * prefix, scatter) produces when its scatter loop runs in order. Values move bit-exactly.
 * ------------------------------------------------------------------------------------- */
void or_csr2csc(int M, int N, const int *rowptr, const int *colind, const float *val,
                int *colptr, int *rowind, float *cscval) {
    int *cursor = (int *)calloc((size_t)N + 1, sizeof(int));
    for (int c = 0; c <= N; ++c) colptr[c] = 0;
    for (int e = 0; e < rowptr[M]; ++e) colptr[colind[e] + 1]++;
    for (int c = 0; c < N; ++c) colptr[c + 1] += colptr[c];
    for (int c = 0; c < N; ++c) cursor[c] = colptr[c];
    for (int m = 0; m < M; ++m)
        for (int e = rowptr[m]; e < rowptr[m + 1]; ++e) {
            const int p = cursor[colind[e]]++;
            rowind[p] = m;
            if (val) cscval[p] = val[e];
        }
    free(cursor);
}

/* Rounding of float to bfloat16 (round to nearest even; NaN kept quiet), returned as the
 * upper 16 bits. Used to build bf16 inputs and the split-bf16 operands on the CPU side. */
uint16_t or_f32_to_bf16(float f) {
    uint32_t u;
    memcpy(&u, &f, 4);
    if ((u & 0x7fffffffu) > 0x7f800000u) return (uint16_t)((u >> 16) | 0x40u);
    const uint32_t lsb = (u >> 16) & 1u;
    u += 0x7fffu + lsb;
    return (uint16_t)(u >> 16);
}

int or_max_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* Unweighted / weighted sum or max aggregation: C[i,:] = reduce over row i of w_e * B[col,:]
 * (w_e = val[e] or 1 when val is NULL), in CSR order: the unweighted sum adds acc += B[...] as
 * the reference's copy-sum kernels do (gcn/pytorch-custom/spmm_kernel.cu:156-173), the
 * weighted sum is the fused chain of rowBaseSpmm3, max takes the rounded product.
 * op: 0 = sum, 1 = max from -inf (fmaxf); both give 0 for rows without entries.
 * op 2 = the reference's DGL copy-max (gcn/dgl-custom/binary_reduce_max.cu): max_init() returns
 * -10000 (:22-24), max_reduce(acc, x) is acc > x ? acc : x (:18-20), applied to each entry of
 * the row in CSR order (topoSimpleSPMMMaxKernel :151-166; the tiled kernels :26-149 apply the
 * same two functions in the same order), and an empty row keeps -10000. */
void or_spmm_reduce_f32(int M, int N, const int *rowptr, const int *colind, const float *val,
                        const float *B, long ldb, float *C, int op) {
    for (int m = 0; m < M; ++m) {
        float *c = C + (long)m * N;
        for (int j = 0; j < N; ++j) c[j] = op == 0 ? 0.0f : op == 1 ? -INFINITY : -10000.0f;
        for (int e = rowptr[m]; e < rowptr[m + 1]; ++e) {
            const float *b = B + (long)colind[e] * ldb;
            for (int j = 0; j < N; ++j) {
                if (op == 0) {
                    c[j] = val ? fmaf(b[j], val[e], c[j]) : c[j] + b[j];
                } else if (op == 1) {
                    c[j] = fmaxf(c[j], val ? val[e] * b[j] : b[j]);
                } else {
                    const float x = val ? val[e] * b[j] : b[j];
                    c[j] = c[j] > x ? c[j] : x;
                }
            }
        }
        if (rowptr[m] == rowptr[m + 1] && op != 2)
            for (int j = 0; j < N; ++j) c[j] = 0.0f;
    }
}

/* Row-pair reuse format of the reference's suitesparse_sdmm.cpp (toDataReuseFormat, :150-179),
 * built from CSR with ascending columns instead of from a dense matrix (the same layout): rows
 * are paired (2p, 2p+1); row 2p's segment lists its entries in column order, each followed by
 * row 2p+1's entry in the same column when there is one (flag 1: it belongs to the next row);
 * row 2p+1's segment keeps its entries in columns row 2p does not have. An unpaired last row is
 * copied. Total entries are unchanged. rowptr2[M+1], colind2/val2/flag2[nnz]. */
void or_csr_to_rowpair(int M, const int *rowptr, const int *colind, const float *val,
                       int *rowptr2, int *colind2, float *val2, unsigned char *flag2) {
    int size = 0;
    for (int r = 0; r < M; ++r) {
        rowptr2[r] = size;
        const int a0 = rowptr[r], a1 = rowptr[r + 1];
        if (r % 2 == 0 && r + 1 < M) {
            const int b1 = rowptr[r + 2];
            int b = rowptr[r + 1];
            for (int e = a0; e < a1; ++e) {
                colind2[size] = colind[e];
                val2[size] = val[e];
                flag2[size] = 0;
                ++size;
                while (b < b1 && colind[b] < colind[e]) ++b;
                if (b < b1 && colind[b] == colind[e]) {
                    colind2[size] = colind[b];
                    val2[size] = val[b];
                    flag2[size] = 1;
                    ++size;
                }
            }
        } else if (r % 2 == 1) {
            const int p0 = rowptr[r - 1], p1 = rowptr[r];
            int q = p0;
            for (int e = a0; e < a1; ++e) {
                while (q < p1 && colind[q] < colind[e]) ++q;
                if (q < p1 && colind[q] == colind[e]) continue; /* moved into row r-1's segment */
                colind2[size] = colind[e];
                val2[size] = val[e];
                flag2[size] = 0;
                ++size;
            }
        } else { /* unpaired last row */
            for (int e = a0; e < a1; ++e) {
                colind2[size] = colind[e];
                val2[size] = val[e];
                flag2[size] = 0;
                ++size;
            }
        }
    }
    rowptr2[M] = size;
}

/* DataReuseSpmm (suitesparse_sdmm.cpp:25-44): for each row m and each entry of its segment,
 * C[m + flag] += val * B[col] by a fused saxpy (one fmaf per column, as OpenBLAS computes
 * it), rows of a pair handled in order (schedule(static, 2)). So row 2p's outputs are the CSR
 * chain, and row 2p+1's chain runs over the entries it shares with row 2p first (in column
 * order), then over its own segment. C is accumulated (the caller zeroes it). */
void or_spmm_rowpair_f32(int M, int N, const int *rowptr2, const int *colind2, const float *val2,
                         const unsigned char *flag2, const float *B, long ldb, float *C, long ldc,
                         int threads) {
#ifdef _OPENMP
    if (threads > 0) omp_set_num_threads(threads);
#pragma omp parallel for schedule(static, 2)
#endif
    for (int m = 0; m < M; ++m) {
        for (int e = rowptr2[m]; e < rowptr2[m + 1]; ++e) {
            float *c = C + (long)(m + flag2[e]) * ldc;
            const float *b = B + (long)colind2[e] * ldb;
            const float v = val2[e];
            for (int j = 0; j < N; ++j) c[j] = fmaf(v, b[j], c[j]);
        }
    }
}
