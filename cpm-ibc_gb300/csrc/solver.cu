// BiCGStab on the device, batched over K slot columns (row-major [D][K]).
//
//   K9   E pass  t = E~ x                          (Interpolation, src/GeneralizedBiCGStabSystem.h:235-261)
//        L pass  y = m x + n (Ldiag x + Loff t)    (LnodiagTimesX/LdiagTimesX/FinalizeMultiplication :65-189)
//        with the BiCGStab dot products fused into the L pass epilogue
//   K10  vector updates of BiCGStab::Solve (src/BiCGStab.h:41-103) fused with
//        their reductions; per-slot scalars stay on the device; reductions are
//        accumulated in FP64 with a fixed-order two-level tree (deterministic
//        and independent of the other slots' contents)
//   K11  mixed precision: the Krylov iteration runs in FP32 (FP32 weights and
//        vectors, FP64 reductions) and is refined in FP64 by reliable updates
//        (Sleijpen & van der Vorst, "Reliable updated residuals in hybrid Bi-CG
//        methods", Computing 56, 1996; the mixed-precision form of Clark et al.,
//        Comput. Phys. Commun. 181, 2010): whenever the FP32 residual has
//        dropped by delta since the last update, or claims convergence, the
//        FP32 solution increment is added to the FP64 solution, the FP64 true
//        residual b - A x replaces the FP32 recursive one and the iteration
//        continues with its search directions; the solve ends when the FP64
//        true residual meets ||b - A x|| <= tol ||b||.
// Every slot is an independent state machine (idle / iterating / refine /
// reliable-update / restart / done), so slots start and finish independently.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <deque>
#include <cstring>
#include <limits>
#include <mutex>
#include <string>

#include "opset.h"

namespace cpm {

enum Phase : int {
    PH_IDLE = 0,
    PH_ITER = 1,
    PH_REFINE = 2,
    PH_DONE = 3,
    PH_RESTART = 4,
    PH_INNER_INIT = 5,
    PH_RELIABLE = 6,
    PH_START = 7  // mixed path: a new right-hand side waiting for k_mixed_start
};

struct Slot {
    double rho, rho_old, alpha, omega, beta;
    double bnorm2, r0norm2, rr, tol2, rr_max;
    double scale, rnorm64, outer_tol2, b64norm2;
    double rr_upd;  // mixed path: FP32 residual norm^2 right after the last reliable update
    double rbest;   // mixed path: smallest FP64 true residual norm so far
    int phase, iters, inner_iters, refinements, restarts, status, krylov_restart;
    int stall;      // mixed path: reliable updates since rbest last improved by 10%
    int fresh;      // mixed path: Krylov space restarted from the FP32 residual, p = r0 = r pending
    int upd_iters;  // mixed path: FP32 iterations since the last reliable update
};

struct SolveParams {
    double tol, delta;
    int max_iters, max_refine, mixed;
    int precond;  // 0 identity, 1 diagonal, 2 damped Jacobi with `sweeps` sweeps
    int sweeps, refine_every;
};

// damping of the Jacobi preconditioner (src/GeneralizedBiCGStabSystem.h:365)
constexpr double JACOBI_OMEGA = 2.0 / 3.0;

constexpr int BS = 256;
constexpr int UNR = 4;       // rows in flight per thread in the row loops
constexpr int RGROUP = 32;   // blocks per first-level group of the grid reduction
constexpr unsigned FULL = 0xffffffffu;

// grid size of the row-loop kernels: UNR rows per thread per trip, at most
// four 256-thread blocks per SM (the reduction tree is fixed by this size)
static inline int sm_count() {
    int dev = 0, sms = 152;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    return sms;
}
static inline int row_grid(int64_t D, int K) {
    const int sms = sm_count();
    const int64_t rpb = BS / K;
    const int64_t need = (D + rpb * UNR - 1) / (rpb * UNR);
    return (int)std::max<int64_t>(1, std::min<int64_t>(need, 4LL * sms));
}
static inline int64_t reduce_groups(int G) { return (G + RGROUP - 1) / RGROUP; }

// ---- per-thread dot products.  FP64 vectors accumulate in FP64.  FP32 vectors
// accumulate in a double-float pair on the FP32 pipes (FP64 units are scarce on
// this GPU): each product a*b is split exactly into p + e by an FMA, p is added
// to the running sum by TwoSum (Knuth), and the rounding errors and e collect
// in the low word, about 48 significant bits in all.  Across threads the
// sums are FP64.
template <class T, int N>
struct Dot;
template <int N>
struct Dot<double, N> {
    double a[N];
    __device__ __forceinline__ Dot() {
#pragma unroll
        for (int d = 0; d < N; ++d) a[d] = 0.0;
    }
    __device__ __forceinline__ void add(int d, double x, double y) { a[d] += x * y; }
    __device__ __forceinline__ void get(double (&o)[N]) const {
#pragma unroll
        for (int d = 0; d < N; ++d) o[d] = a[d];
    }
};
template <int N>
struct Dot<float, N> {
    float hi[N], lo[N];
    __device__ __forceinline__ Dot() {
#pragma unroll
        for (int d = 0; d < N; ++d) hi[d] = lo[d] = 0.0f;
    }
    __device__ __forceinline__ void add(int d, float x, float y) {
        const float p = __fmul_rn(x, y);
        const float e = __fmaf_rn(x, y, -p);  // x*y = p + e exactly
        const float s = __fadd_rn(hi[d], p);
        const float bp = __fsub_rn(s, hi[d]);
        const float err = __fadd_rn(__fsub_rn(hi[d], __fsub_rn(s, bp)), __fsub_rn(p, bp));  // hi + p = s + err
        hi[d] = s;
        lo[d] = __fadd_rn(lo[d], __fadd_rn(err, e));
    }
    __device__ __forceinline__ void get(double (&o)[N]) const {
#pragma unroll
        for (int d = 0; d < N; ++d) o[d] = (double)hi[d] + (double)lo[d];
    }
};

// ---- fixed-order grid reduction of NDOT FP64 sums per slot.  Blocks reduce
// their rows with a tree, groups of RGROUP blocks are summed in block order by
// the group's last block, and the groups in group order by the last group: the
// result depends only on the grid size, never on timing or on other slots.
// partial holds (G + groups) * K * NDOT doubles, counter 1 + groups zeros.
// SUMMED: the block's per-slot sums are already in v of threads tid < K (the
// other threads' v are not read), and the block tree is skipped.
template <int K, int NDOT, bool SUMMED = false>
__device__ __forceinline__ bool grid_reduce(double (&v)[NDOT], double *partial, unsigned int *counter, double (&out)[NDOT]) {
    __shared__ double sh[NDOT][BS];
    __shared__ bool last;
    const int tid = threadIdx.x;
    constexpr int RPB = BS / K;
    const int slot = tid % K, chunk = tid / K;
    auto tree = [&]() {
        __syncthreads();
        for (int h = RPB / 2; h > 0; h >>= 1) {
            if (chunk < h)
#pragma unroll
                for (int d = 0; d < NDOT; ++d) sh[d][tid] += sh[d][tid + h * K];
            __syncthreads();
        }
    };
    if (SUMMED) {
        if (tid < K)
#pragma unroll
            for (int d = 0; d < NDOT; ++d) sh[d][tid] = v[d];
        __syncthreads();
    } else {
#pragma unroll
        for (int d = 0; d < NDOT; ++d) sh[d][tid] = v[d];
        tree();
    }
    const unsigned G = gridDim.x, grp = blockIdx.x / RGROUP, ngrp = (G + RGROUP - 1) / RGROUP;
    double *gpart = partial + (size_t)G * K * NDOT;
    if (tid < K)
#pragma unroll
        for (int d = 0; d < NDOT; ++d) partial[((size_t)blockIdx.x * K + tid) * NDOT + d] = sh[d][tid];
    __threadfence();
    __syncthreads();
    const unsigned b0 = grp * RGROUP, b1 = min(b0 + RGROUP, G);
    if (tid == 0) last = (atomicAdd(counter + 1 + grp, 1u) == b1 - b0 - 1);
    __syncthreads();
    if (!last) return false;
    __threadfence();
    double acc[NDOT];
#pragma unroll
    for (int d = 0; d < NDOT; ++d) acc[d] = 0.0;
#pragma unroll
    for (int q = 0; q < (RGROUP + RPB - 1) / RPB; ++q) {
        const unsigned b = b0 + chunk + q * RPB;
        if (b < b1)
#pragma unroll
            for (int d = 0; d < NDOT; ++d) acc[d] += __ldcg(partial + ((size_t)b * K + slot) * NDOT + d);
    }
#pragma unroll
    for (int d = 0; d < NDOT; ++d) sh[d][tid] = acc[d];
    tree();
    if (tid < K)
#pragma unroll
        for (int d = 0; d < NDOT; ++d) gpart[((size_t)grp * K + tid) * NDOT + d] = sh[d][tid];
    if (tid == 0) counter[1 + grp] = 0u;
    __threadfence();
    __syncthreads();
    if (tid == 0) last = (atomicAdd(counter, 1u) == ngrp - 1);
    __syncthreads();
    if (!last) return false;
    __threadfence();
#pragma unroll
    for (int d = 0; d < NDOT; ++d) acc[d] = 0.0;
    for (unsigned g = chunk; g < ngrp; g += RPB)
#pragma unroll
        for (int d = 0; d < NDOT; ++d) acc[d] += __ldcg(gpart + ((size_t)g * K + slot) * NDOT + d);
#pragma unroll
    for (int d = 0; d < NDOT; ++d) sh[d][tid] = acc[d];
    tree();
    if (tid < K)
#pragma unroll
        for (int d = 0; d < NDOT; ++d) out[d] = sh[d][tid];
    if (tid == 0) *counter = 0u;
    return tid < K;
}

// ---- per-slot scalar updates at the end of a reduction (one thread per slot)

// alpha = rho / (r0 . v)   (src/BiCGStab.h:79-80)
template <class T>
__device__ __forceinline__ void alpha_update(Slot &S, double r0v) {
    if (S.phase != PH_ITER) return;
    S.fresh = 0;  // k_update_p has consumed it
    S.alpha = S.rho / r0v;
    if constexpr (sizeof(T) == 4) {
        // FP32 inner iteration: r0 . v = 0 (or a non-finite value) ends this
        // Krylov space; the FP64 reliable update restarts it from the true residual
        if (!isfinite(S.alpha)) {
            S.krylov_restart = 1;
            S.rho_old = S.rho;
            S.phase = PH_REFINE;
        }
    }
}

// omega = (t . s) / (t . t)   (src/BiCGStab.h:85-95)
__device__ __forceinline__ void omega_update(Slot &S, double tt, double ts) {
    if (S.phase != PH_ITER) return;
    S.omega = (tt > 0.0) ? ts / tt : 0.0;
}

// r . r and r0 . r: convergence test, rho, beta   (src/BiCGStab.h:97-103, :59-73)
__device__ __forceinline__ void xr_update(Slot &S, const SolveParams &P, double rr, double r0r) {
    if (S.phase != PH_ITER) return;
    S.iters += 1;
    S.inner_iters += 1;
    S.upd_iters += 1;
    S.rr = rr;
    const bool conv = S.rr <= S.tol2;  // false for a non-finite residual
    if (P.mixed) {
        S.rr_max = fmax(S.rr_max, S.rr);
        // a slot whose FP32 residual claims convergence waits for the next
        // reliable update; one whose residual merely fell by delta keeps
        // iterating until then (k_refine_gate)
        if (conv || S.iters >= P.max_iters || !isfinite(S.rr)) {
            S.rho_old = S.rho;
            S.phase = PH_REFINE;
            return;
        }
        // an FP32 residual 10^4 times larger than right after the last
        // reliable update has diverged (BiCGStab residuals may spike by
        // a few orders of magnitude and recover; this does not): restart
        // the Krylov space from the FP64 true residual
        if (S.rr > 1e8 * S.rr_upd) {
            S.krylov_restart = 1;
            S.rho_old = S.rho;
            S.phase = PH_REFINE;
            return;
        }
    } else {
        if (conv) {
            S.phase = PH_DONE;
            S.status = 0;
            return;
        }
        if (S.iters >= P.max_iters || !isfinite(S.rr)) {
            S.phase = PH_DONE;
            S.status = isfinite(S.rr) ? CPM_ERR_NOT_CONVERGED : CPM_ERR_BREAKDOWN;
            return;
        }
    }
    S.rho_old = S.rho;
    S.rho = r0r;
    const double eps = 2.220446049250313e-16;
    if (fabs(S.rho) < eps * eps * S.r0norm2) {  // restart on rho breakdown (src/BiCGStab.h:62-71)
        if (P.mixed) {
            // FP32 iteration: restart in place from the recurrence residual
            // (r0 = p = r in k_update_p, rho = r . r) rather than idle until the
            // next reliable update
            S.fresh = 1;
            S.restarts += 1;
            S.r0norm2 = S.rr;
            S.rho = S.rr;
            S.rho_old = 1.0;
            S.alpha = 1.0;
            S.omega = 1.0;
            S.beta = S.rr;
        } else {
            S.phase = PH_RESTART;
        }
        return;
    }
    S.beta = (S.rho / S.rho_old) * (S.alpha / S.omega);
}

// ================================================================= kernels

// 32 slots, plane-split: one 4-warp block per base group (grid-stride), then
// identity rows copied warp per row.  ph < 0: every slot.
template <class T>
__global__ void __launch_bounds__(128) k_epass32s(OpView<T> op, const Slot *__restrict__ sl, int ph, const T *__restrict__ x,
                                                  T *__restrict__ t) {
    __shared__ EGShared<T> sh;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const bool act = (ph < 0) || sl[lane].phase == ph;
    if (!__any_sync(FULL, act)) return;  // the same 32 slots in every warp: block-uniform
    for (int64_t g = blockIdx.x; g < op.n_grp; g += gridDim.x) {
        int col[16];
        T xb[16];
        e_group_cols(op.gcols, g, warp, col);
        e_group_x(x, col, lane, act, xb);
        e_group_split<T>(op, op.grp[g], op.grp[g + 1], warp, lane, act, sh, xb, t);
    }
    if (act)
        for (int64_t q = (int64_t)blockIdx.x * 4 + warp; q < op.n_ident; q += (int64_t)gridDim.x * 4) {
            const uint32_t r = (uint32_t)op.ident[q];
            t[r * 32u + lane] = x[r * 32u + lane];
        }
}

// IBC patch of one row of a 32-slot E pass (warp per row, lane = slot): patch-
// list row q's value from its bulk value acc, sign (acc + sum_e w_e (x[new_e] -
// x[old_e])) + xval x[xcol]: moved stencil points read the IBC DOF column
// instead of the tube node (IBCMatrixManipulations::AddIBCExtension's column
// moves, src/IBCMatrixManipulations.cpp:118-186); a point that moves to
// several IBCs adds w x[target] for each further IBC (OpView::ov_*).  The lanes load 32 entries at
// once and broadcast them, so a row's x loads are all in flight together.
// q is the same in every lane; inactive slots (act false) load nothing.
template <class T>
__device__ __forceinline__ T ovl_e_patch(const int32_t *patch, const int32_t *ov_ptr, const int32_t *ov_col, const T *ov_w,
                                         uint32_t r, T acc, int lane, bool act, const T *__restrict__ x) {
    const int pi = patch[r];
    for (int e = ov_ptr[2 * pi]; e < ov_ptr[2 * pi + 1]; ++e)
        acc = fma_rn(ov_w[e], act ? x[(uint32_t)ov_col[e] * 32u + lane] : T(0), acc);
    return acc;
}

template <class T, bool OVL>
__device__ __forceinline__ T patch_row(const OpView<T> &op, int q, uint32_t r, T acc, int lane, bool act,
                                       const T *__restrict__ x) {
    const int e0 = op.pl_off[q], e1 = op.pl_off[q + 1], xc = op.pl_xcol[q], neg = op.pl_neg[q];
    const T xv = op.pl_xval[q];
    const T xe = (act && xc >= 0) ? x[(uint32_t)xc * 32u + lane] : T(0);
    for (int base = e0; base < e1; base += 32) {
        const int cnt = min(32, e1 - base);
        int nc = 0, oc = 0;
        T w = 0;
        if (lane < cnt) {
            nc = op.pe_new[base + lane];
            oc = op.pe_old[base + lane];
            w = op.pe_w[base + lane];
        }
        for (int u0 = 0; u0 < cnt; u0 += 8) {
            T xn[8], xo[8], ww[8];
#pragma unroll
            for (int u = 0; u < 8; ++u) {
                const int k = u0 + u;
                const uint32_t ncu = (uint32_t)__shfl_sync(FULL, nc, k & 31), ocu = (uint32_t)__shfl_sync(FULL, oc, k & 31);
                ww[u] = __shfl_sync(FULL, w, k & 31);
                const bool ok = act && k < cnt;
                xn[u] = ok ? x[ncu * 32u + lane] : T(0);
                xo[u] = ok ? x[ocu * 32u + lane] : T(0);
            }
#pragma unroll
            for (int u = 0; u < 8; ++u)
                if (u0 + u < cnt) acc = fma_rn(ww[u], sub_rn(xn[u], xo[u]), acc);
        }
    }
    if constexpr (OVL)
        if (neg & 2) acc = ovl_e_patch<T>(op.patch, op.ov_ptr, op.ov_col, op.ov_w, r, acc, lane, act, x);
    if (neg & 1) acc = -acc;
    if (xc >= 0) acc = fma_rn(xv, xe, acc);
    return acc;
}

// 32 FP32 slots, warp per base group: the warp gathers the group's 64 x
// values plane by plane (16 columns each) and keeps each pair of rows' sum in
// registers (f32x2): plane i adds wx_i (sum_j wy_j sum_k wz_k x_ijk) in the
// plane order of k_epass32s's combine, so the results are the same bit for
// bit, with no block-level synchronisation and no shared partial sums.  Rows
// EW_ROWS at a time; weights staged pair-interleaved in the warp's shared
// memory.  Identity rows copied warp per row.  ph < 0: every slot.
constexpr int EW_ROWS = 8;
__global__ void __launch_bounds__(128) k_epass32w(OpView<float> op, const Slot *__restrict__ sl, int ph,
                                                  const float *__restrict__ x, float *__restrict__ t) {
    __shared__ __align__(16) float sw[4][EW_ROWS * 12];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const bool act = (ph < 0) || sl[lane].phase == ph;
    if (!__any_sync(FULL, act)) return;  // the same 32 slots in every warp: block-uniform
    float *w = sw[warp];
    const float *__restrict__ xl = x + lane;
    const int64_t W = (int64_t)gridDim.x * 4;
    for (int64_t g = (int64_t)blockIdx.x * 4 + warp; g < op.n_grp; g += W) {
        const int p0 = op.grp[g], p1 = op.grp[g + 1];
        for (int c0 = p0; c0 < p1; c0 += EW_ROWS) {
            // rows in pairs, the odd row of a last pair with zero weights
            const int nr = min(p1 - c0, EW_ROWS), np = (nr + 1) >> 1;
            __syncwarp();
            for (int e = lane; e < 24 * np; e += 32) {
                const int q = e / 12, c = e - 12 * q;
                w[24 * (q >> 1) + 2 * c + (q & 1)] = q < nr ? op.w_ord[12 * (size_t)(c0 + q) + c] : 0.f;
            }
            const int row = lane < nr ? op.ord[c0 + lane] : 0;  // lane q: row q of the chunk
            __syncwarp();
            uint64_t acc[EW_ROWS / 2];
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                int col[16];
                float xb[16];
                e_group_cols(op.gcols, g, i, col);
                // every lane loads (inactive slots' values are computed and not stored);
                // the rows are whole 128-byte lines either way
#pragma unroll
                for (int q = 0; q < 16; ++q) xb[q] = xl[(uint32_t)col[q] * 32u];
                uint64_t x2[16];
#pragma unroll
                for (int q = 0; q < 16; ++q) x2[q] = f2_pack(xb[q], xb[q]);
#pragma unroll
                for (int p = 0; p < EW_ROWS / 2; ++p)
                    if (p < np) {
                        const float *wp = w + 24 * p;
                        const uint64_t wx2 = *(const uint64_t *)(wp + 2 * i);
                        const ulonglong2 y01 = *(const ulonglong2 *)(wp + 8), y23 = *(const ulonglong2 *)(wp + 12);
                        const ulonglong2 z01 = *(const ulonglong2 *)(wp + 16), z23 = *(const ulonglong2 *)(wp + 20);
                        const uint64_t wy2[4] = {y01.x, y01.y, y23.x, y23.y}, wz2[4] = {z01.x, z01.y, z23.x, z23.y};
                        uint64_t ay2 = 0ull;
#pragma unroll
                        for (int j = 0; j < 4; ++j) {
                            uint64_t az2 = f2_mul(wz2[0], x2[4 * j]);
                            az2 = f2_fma(wz2[1], x2[4 * j + 1], az2);
                            az2 = f2_fma(wz2[2], x2[4 * j + 2], az2);
                            az2 = f2_fma(wz2[3], x2[4 * j + 3], az2);
                            ay2 = j == 0 ? f2_mul(wy2[0], az2) : f2_fma(wy2[j], az2, ay2);
                        }
                        const uint64_t part = f2_mul(wx2, ay2);
                        acc[p] = i == 0 ? part : f2_add(acc[p], part);
                    }
            }
#pragma unroll
            for (int p = 0; p < EW_ROWS / 2; ++p)
                if (2 * p < nr) {
                    float lo, hi;
                    f2_unpack(acc[p], lo, hi);
                    const int r0 = __shfl_sync(FULL, row, 2 * p), r1 = __shfl_sync(FULL, row, 2 * p + 1);
                    if (act) {
                        t[(uint32_t)r0 * 32u + lane] = lo;
                        if (2 * p + 1 < nr) t[(uint32_t)r1 * 32u + lane] = hi;
                    }
                }
        }
    }
    if (act)
        for (int64_t q = (int64_t)blockIdx.x * 4 + warp; q < op.n_ident; q += W) {
            const uint32_t r = (uint32_t)op.ident[q];
            t[r * 32u + lane] = x[r * 32u + lane];
        }
}

// 1 slot: one thread per row, rows visited in base-point order so that the
// threads of a warp that share a base read the same cache lines.
template <class T>
__global__ void k_epass1(OpView<T> op, const Slot *__restrict__ sl, int ph, const T *__restrict__ x, T *__restrict__ t) {
    if (ph >= 0 && sl[0].phase != ph) return;
    const int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (p < op.n_ord) {
        const int64_t r = op.ord[p];
        t[r] = e_row_thread<T, 1>(op, r, 0, x);
        return;
    }
    const int64_t q = p - op.n_ord;
    if (q < op.n_ident) {
        const int64_t r = op.ident[q];
        t[r] = x[r];
    }
}

// the patch as a pass of its own after the bulk 32-slot E pass, warp per
// patch-list row (consecutive rows on neighbouring warps, whose gathers share
// cache lines)
template <class T, bool OVL>
__global__ void __launch_bounds__(128) k_epatch32(OpView<T> op, const Slot *__restrict__ sl, int ph, const T *__restrict__ x,
                                                  T *__restrict__ t) {
    const int lane = threadIdx.x & 31;
    const bool act = (ph < 0) || sl[lane].phase == ph;
    if (!__any_sync(FULL, act)) return;  // the same slots in every warp: block-uniform
    const int64_t warps = (int64_t)gridDim.x * 4;
    for (int64_t q = (int64_t)blockIdx.x * 4 + (threadIdx.x >> 5); q < op.n_pl; q += warps) {
        const uint32_t r = (uint32_t)op.pl_row[q];
        const T acc = act ? t[r * 32u + lane] : T(0);
        const T v = patch_row<T, OVL>(op, (int)q, r, acc, lane, act, x);
        if (act) t[r * 32u + lane] = v;
    }
}

// per-slot E corrections of a batch with one point IBC per slot (OpView::sp_*),
// after the bulk E pass: warp per row with records, lane = slot,
// t += sum over the slot's E entries of w (x[DOF column] - x[replaced column])
template <class T>
__global__ void __launch_bounds__(128) k_slot_epatch32(OpView<T> op, const Slot *__restrict__ sl, int ph, const T *__restrict__ x,
                                                       T *__restrict__ t) {
    const int lane = threadIdx.x & 31;
    const bool act = (ph < 0) || sl[lane].phase == ph;
    if (!__any_sync(FULL, act)) return;
    const int64_t warps = (int64_t)gridDim.x * 4;
    for (int64_t q = (int64_t)blockIdx.x * 4 + (threadIdx.x >> 5); q < op.n_sp_rows; q += warps) {
        const int64_t r = op.sp_rows[q];
        T c = 0;
        bool any = false;
        for (int e = op.sp_ptr[r]; e < op.sp_ptr[r + 1]; ++e) {
            const int4 rec = op.sp_rec[e];
            if (rec.x == lane && rec.y == 0) {
                c += op.sp_w[e] * (x[(int64_t)rec.w * 32 + lane] - x[(int64_t)rec.z * 32 + lane]);
                any = true;
            }
        }
        if (act && any) t[r * 32 + lane] += c;
    }
}

template <class T>
static void slot_epatch(const OpView<T> &op, const Slot *sl, int ph, const T *x, T *t, cudaStream_t st) {
    const int64_t blocks = std::max<int64_t>(1, std::min<int64_t>((op.n_sp_rows + 3) / 4, 16LL * sm_count()));
    k_slot_epatch32<T><<<(unsigned)blocks, 128, 0, st>>>(op, sl, ph, x, t);
}

// default launch shapes of the 32-slot E passes (blocks per SM caps of the
// grid-stride loops): the FP32 bulk pass's best on the sphere with two circles at
// dx 0.025; for the patch and FP64 passes the autotuner chose 64 or more blocks
// per SM on the sphere, the torus and the mesh of the serving stream
constexpr int E32_BPS = 32, PATCH_BPS = 64, E64_BPS = 64;

// kernels one E pass of x launches
template <class T, int K>
static inline int epass_kernels(const OpView<T> &op, const T *) {
    const int sp = (K == 32 && op.n_sp_rows > 0) ? 1 : 0;
    return ((K == 32 && op.n_pl > 0) ? 2 : 1) + sp;
}

template <class T, int K>
static void launch_epass(const OpView<T> &op, const Slot *sl, int ph, const T *x, T *t, cudaStream_t st) {
    static_assert(K == 1 || K == 32, "slot widths 1 and 32");
    if constexpr (K == 32) {
        if constexpr (sizeof(T) == 4) {
            const int64_t bps = op.e32_bps > 0 ? op.e32_bps : E32_BPS;
            const int64_t blocks = std::max<int64_t>(1, std::min<int64_t>((op.n_grp + 3) / 4, bps * sm_count()));
            k_epass32w<<<(unsigned)blocks, 128, 0, st>>>(op, sl, ph, x, t);
        } else {
            const int64_t bps = op.e64_bps > 0 ? op.e64_bps : E64_BPS;
            const int64_t blocks = std::max<int64_t>(1, std::min<int64_t>(op.n_grp, bps * sm_count()));
            k_epass32s<T><<<(unsigned)blocks, 128, 0, st>>>(op, sl, ph, x, t);
        }
    } else {
        const int64_t threads = op.n_ord + op.n_ident;
        k_epass1<T><<<(unsigned)((threads + BS - 1) / BS), BS, 0, st>>>(op, sl, ph, x, t);
    }
    if (K == 32 && op.n_pl > 0) {  // the gather passes correct the IBC patch rows afterwards
        const int64_t bps = op.patch_bps > 0 ? op.patch_bps : PATCH_BPS;
        const int64_t blocks = std::max<int64_t>(1, std::min<int64_t>((op.n_pl + 3) / 4, bps * sm_count()));
        if (op.ov_ptr)
            k_epatch32<T, true><<<(unsigned)blocks, 128, 0, st>>>(op, sl, ph, x, t);
        else
            k_epatch32<T, false><<<(unsigned)blocks, 128, 0, st>>>(op, sl, ph, x, t);
    }
    if (K == 32 && op.n_sp_rows > 0) slot_epatch(op, sl, ph, x, t, st);
}

int epass64_batch(const cpm_opset_s *o, bool slot_patches, const double *x, double *t) {
    OpView<double> v = o->view<double>();
    if (!slot_patches) {
        v.sp_ptr = nullptr;
        v.n_sp_rows = 0;
    }
    launch_epass<double, 32>(v, nullptr, -1, x, t, stream());
    count_launches(epass_kernels<double, 32>(v, x));
    CPM_CUDA_TRY(cudaGetLastError());
    return 0;
}

// Row loops: thread (row group, slot s) with K slots per row; each trip
// handles UNR rows rb + u * rstride, all of whose loads are issued first.
#define GRID_LOOP                                                    \
    constexpr int RPB = BS / K;                                      \
    const int s = threadIdx.x % K;                                   \
    const int64_t r0i = (int64_t)blockIdx.x * RPB + threadIdx.x / K; \
    const int64_t rstride = (int64_t)gridDim.x * RPB;
#define ROWS_UNR_N(Dn, UN) for (int64_t rb = r0i; rb < (Dn); rb += (int64_t)(UN) * rstride)
#define ROWS_OF_TRIP_N(rr, UN)                                        \
    int64_t rr[UN];                                                   \
    _Pragma("unroll") for (int u = 0; u < (UN); ++u) rr[u] = rb + (int64_t)u * rstride;
#define ROWS_UNR(Dn) ROWS_UNR_N(Dn, UNR)
#define ROWS_OF_TRIP(rr) ROWS_OF_TRIP_N(rr, UNR)
// FP64 streams of six vectors keep two rows in flight within 64 registers
template <class T>
constexpr int unr_stream6() { return sizeof(T) == 8 ? 2 : UNR; }

// y = m x + n (Ldiag x + Loff E~-gathered neighbours): the L pass of one apply
template <class T, int K>
__global__ void __launch_bounds__(BS, 4) k_lpass(OpView<T> op, T m, T n, const T *__restrict__ x, const T *__restrict__ t,
                                              T *__restrict__ y) {
    GRID_LOOP
    ROWS_UNR(op.D) {
        ROWS_OF_TRIP(rr)
        T v[UNR];
        l_rows<T, K, UNR>(op, rr, s, m, n, x, t, true, v);
#pragma unroll
        for (int u = 0; u < UNR; ++u)
            if (rr[u] < op.D) y[rr[u] * K + s] = v[u];
    }
}

// --- start of a (plain or mixed) Krylov iteration: x = 0, r = r0 = rhs, p = v = 0
// rhs = b (plain) or (T)(r64 / scale) (mixed)
template <class T, int K>
__global__ void __launch_bounds__(BS, 4) k_init(OpView<T> op, Slot *sl, SolveParams P, int from_phase, const double *__restrict__ rhs64,
                       T *__restrict__ x, T *__restrict__ r, T *__restrict__ r0, T *__restrict__ p, T *__restrict__ v,
                       double *partial, unsigned int *counter) {
    GRID_LOOP
    const bool act = sl[s].phase == from_phase;
    const double inv = (from_phase == PH_INNER_INIT) ? 1.0 / sl[s].scale : 1.0;
    Dot<T, 1> acc;
    if (act)
        ROWS_UNR(op.D) {
            ROWS_OF_TRIP(rr)
            double bb[UNR];
#pragma unroll
            for (int u = 0; u < UNR; ++u) bb[u] = rr[u] < op.D ? rhs64[rr[u] * K + s] : 0.0;
#pragma unroll
            for (int u = 0; u < UNR; ++u)
                if (rr[u] < op.D) {
                    const int64_t i = rr[u] * K + s;
                    T bv = (T)(bb[u] * inv);
                    x[i] = 0;
                    r[i] = bv;
                    r0[i] = bv;
                    p[i] = 0;
                    v[i] = 0;
                    acc.add(0, bv, bv);
                }
        }
    double av[1], tot[1];
    acc.get(av);
    if (grid_reduce<K, 1>(av, partial, counter, tot)) {
        Slot &S = sl[threadIdx.x];
        if (S.phase != from_phase) return;
        double b2 = tot[0];
        S.bnorm2 = b2;
        S.r0norm2 = b2;
        S.rr = b2;
        S.rr_max = b2;
        S.rr_upd = b2;
        S.rho_old = 1.0;
        S.alpha = 1.0;
        S.omega = 1.0;
        S.inner_iters = 0;
        S.upd_iters = 0;
        S.krylov_restart = 0;
        if (from_phase == PH_INNER_INIT) {
            // claimed convergence of the FP32 residual, in the scaled system
            S.tol2 = P.tol * P.tol * S.b64norm2 / (S.scale * S.scale);
        } else {
            S.tol2 = P.tol * P.tol * b2;  // BiCGStab::Solve: tol2 = tol^2 ||b||^2 (src/BiCGStab.h:56)
            S.iters = 0;
            S.restarts = 0;
            S.refinements = 0;
        }
        if (!isfinite(b2)) {  // a non-finite right-hand side never counts as converged
            S.phase = PH_DONE;
            S.status = CPM_ERR_BREAKDOWN;
            return;
        }
        if (b2 == 0.0) {  // src/BiCGStab.h:53: x = 0, converged
            S.phase = (from_phase == PH_INNER_INIT) ? PH_REFINE : PH_DONE;
            S.status = 0;
            return;
        }
        if (S.rr <= S.tol2) {
            S.phase = (from_phase == PH_INNER_INIT) ? PH_REFINE : PH_DONE;
            return;
        }
        S.rho = b2;  // r0 . r for the first iteration
        S.beta = (S.rho / S.rho_old) * (S.alpha / S.omega);
        S.phase = PH_ITER;
    }
}

// p = (p - w v) beta + r ; y = M^-1 p   (src/BiCGStab.h:74-78)
// M^-1 here is the diagonal inverse (ys = 1, pden = m + n L_rr), the identity
// (pden = null) or the first Jacobi sweep from zero, y = omega (p / pden)
// (src/GeneralizedBiCGStabSystem.h:358-377 with result = 0 and A 0 = 0)
template <class T, int K>
__global__ void __launch_bounds__(BS, 4) k_update_p(int64_t D, const Slot *__restrict__ sl, const T *__restrict__ pden, T ys,
                                                 const T *__restrict__ r, const T *__restrict__ v, T *__restrict__ p,
                                                 T *__restrict__ y, T *__restrict__ r0) {
    GRID_LOOP
    constexpr int UN = unr_stream6<T>();
    if (sl[s].phase != PH_ITER) return;
    const T w = (T)sl[s].omega, beta = (T)sl[s].beta;
    const bool fresh = sl[s].fresh;  // restarted Krylov space: p = r0 = r
    ROWS_UNR_N(D, UN) {
        ROWS_OF_TRIP_N(rr, UN)
        T pv[UN], vv[UN], rv[UN], dv[UN];
#pragma unroll
        for (int u = 0; u < UN; ++u)
            if (rr[u] < D) {
                const int64_t i = rr[u] * K + s;
                pv[u] = p[i];
                vv[u] = v[i];
                rv[u] = r[i];
                dv[u] = pden ? pden[rr[u]] : T(1);
            }
#pragma unroll
        for (int u = 0; u < UN; ++u)
            if (rr[u] < D) {
                const int64_t i = rr[u] * K + s;
                T pi = -w * vv[u] + pv[u];
                pi *= beta;
                pi = pi + rv[u];
                if (fresh) {
                    pi = rv[u];
                    r0[i] = pi;
                }
                p[i] = pi;
                y[i] = pden ? ys * (pi / dv[u]) : pi;
            }
    }
}

// v = A y with r0 . v  ->  alpha = rho / (r0 . v)   (src/BiCGStab.h:79-80)
template <class T, int K>
__global__ void __launch_bounds__(BS, 4) k_apply_alpha(OpView<T> op, Slot *sl, T m, T n, const T *__restrict__ y,
                                                    const T *__restrict__ te, const T *__restrict__ r0, T *__restrict__ v,
                                                    double *partial, unsigned int *counter) {
    GRID_LOOP
    const bool act = sl[s].phase == PH_ITER;
    Dot<T, 1> acc;
    if (act)
        ROWS_UNR(op.D) {
            ROWS_OF_TRIP(rr)
            T r0v[UNR], vv[UNR];
#pragma unroll
            for (int u = 0; u < UNR; ++u) r0v[u] = rr[u] < op.D ? r0[rr[u] * K + s] : T(0);
            l_rows<T, K, UNR>(op, rr, s, m, n, y, te, true, vv);
#pragma unroll
            for (int u = 0; u < UNR; ++u)
                if (rr[u] < op.D) {
                    v[rr[u] * K + s] = vv[u];
                    acc.add(0, r0v[u], vv[u]);
                }
        }
    double av[1], tot[1];
    acc.get(av);
    if (grid_reduce<K, 1>(av, partial, counter, tot)) alpha_update<T>(sl[threadIdx.x], tot[0]);
}

// s = r - alpha v ; z = M^-1 s   (src/BiCGStab.h:82-84), M^-1 as in k_update_p
template <class T, int K>
__global__ void __launch_bounds__(BS, 4) k_update_s(int64_t D, const Slot *__restrict__ sl, const T *__restrict__ pden, T ys,
                                                 const T *__restrict__ r, const T *__restrict__ v, T *__restrict__ sv,
                                                 T *__restrict__ z) {
    GRID_LOOP
    if (sl[s].phase != PH_ITER) return;
    const T a = (T)sl[s].alpha;
    ROWS_UNR(D) {
        ROWS_OF_TRIP(rr)
        T vv[UNR], rv[UNR], dv[UNR];
#pragma unroll
        for (int u = 0; u < UNR; ++u)
            if (rr[u] < D) {
                const int64_t i = rr[u] * K + s;
                vv[u] = v[i];
                rv[u] = r[i];
                dv[u] = pden ? pden[rr[u]] : T(1);
            }
#pragma unroll
        for (int u = 0; u < UNR; ++u)
            if (rr[u] < D) {
                const int64_t i = rr[u] * K + s;
                T si = -a * vv[u] + rv[u];
                sv[i] = si;
                z[i] = pden ? ys * (si / dv[u]) : si;
            }
    }
}

// one further damped Jacobi sweep on A y = c, after the E pass te = E~ y:
// y += omega ((c - A y) / pden)   (src/GeneralizedBiCGStabSystem.h:366-376).
// Row r of A y reads y only at row r, so the update is in place.
template <class T, int K>
__global__ void __launch_bounds__(BS, 4) k_jacobi_sweep(OpView<T> op, const Slot *__restrict__ sl, T m, T n,
                                                     const T *__restrict__ c, const T *__restrict__ te,
                                                     const T *__restrict__ pden, T omega, T *y) {
    GRID_LOOP
    if (sl[s].phase != PH_ITER) return;
    ROWS_UNR(op.D) {
        ROWS_OF_TRIP(rr)
        T cv[UNR], dv[UNR], ay[UNR];
#pragma unroll
        for (int u = 0; u < UNR; ++u)
            if (rr[u] < op.D) {
                cv[u] = c[rr[u] * K + s];
                dv[u] = pden[rr[u]];
            }
        l_rows<T, K, UNR>(op, rr, s, m, n, y, te, true, ay);
#pragma unroll
        for (int u = 0; u < UNR; ++u)
            if (rr[u] < op.D) {
                const int64_t i = rr[u] * K + s;
                y[i] = y[i] + omega * ((cv[u] - ay[u]) / dv[u]);
            }
    }
}

// t = A z with t.t and t.s  ->  omega   (src/BiCGStab.h:85-95)
template <class T, int K>
__global__ void __launch_bounds__(BS, 4) k_apply_omega(OpView<T> op, Slot *sl, T m, T n, const T *__restrict__ z,
                                                    const T *__restrict__ te, const T *__restrict__ sv, T *__restrict__ tv,
                                                    double *partial, unsigned int *counter) {
    GRID_LOOP
    const bool act = sl[s].phase == PH_ITER;
    Dot<T, 2> acc;
    if (act)
        ROWS_UNR(op.D) {
            ROWS_OF_TRIP(rr)
            T svv[UNR], tt[UNR];
#pragma unroll
            for (int u = 0; u < UNR; ++u) svv[u] = rr[u] < op.D ? sv[rr[u] * K + s] : T(0);
            l_rows<T, K, UNR>(op, rr, s, m, n, z, te, true, tt);
#pragma unroll
            for (int u = 0; u < UNR; ++u)
                if (rr[u] < op.D) {
                    tv[rr[u] * K + s] = tt[u];
                    acc.add(0, tt[u], tt[u]);
                    acc.add(1, tt[u], svv[u]);
                }
        }
    double av[2], tot[2];
    acc.get(av);
    if (grid_reduce<K, 2>(av, partial, counter, tot)) omega_update(sl[threadIdx.x], tot[0], tot[1]);
}

// x += alpha y + w z ; r = s - w t ; r.r and r0.r -> convergence test, rho, beta
// (src/BiCGStab.h:97-103 and the loop head :59-73)
template <class T, int K>
__global__ void __launch_bounds__(BS, 4) k_update_xr(int64_t D, Slot *sl, SolveParams P, const T *__restrict__ y,
                                                  const T *__restrict__ z, const T *__restrict__ sv,
                                                  const T *__restrict__ tv, const T *__restrict__ r0, T *__restrict__ x,
                                                  T *__restrict__ r, double *partial, unsigned int *counter) {
    GRID_LOOP
    const bool act = sl[s].phase == PH_ITER;
    Dot<T, 2> acc;
    if (act) {
        const T a = (T)sl[s].alpha, w = (T)sl[s].omega;
        constexpr int UN = unr_stream6<T>();
        ROWS_UNR_N(D, UN) {
            ROWS_OF_TRIP_N(rr, UN)
            T yv[UN], zv[UN], xv[UN], tw[UN], sw[UN], r0v[UN];
#pragma unroll
            for (int u = 0; u < UN; ++u)
                if (rr[u] < D) {
                    const int64_t i = rr[u] * K + s;
                    yv[u] = y[i];
                    zv[u] = z[i];
                    xv[u] = x[i];
                    tw[u] = tv[i];
                    sw[u] = sv[i];
                    r0v[u] = r0[i];
                }
#pragma unroll
            for (int u = 0; u < UN; ++u)
                if (rr[u] < D) {
                    const int64_t i = rr[u] * K + s;
                    T xi = a * yv[u] + xv[u];
                    x[i] = w * zv[u] + xi;
                    T ri = -w * tw[u] + sw[u];
                    r[i] = ri;
                    acc.add(0, ri, ri);
                    acc.add(1, r0v[u], ri);
                }
        }
    }
    double av[2], tot[2];
    acc.get(av);
    if (grid_reduce<K, 2>(av, partial, counter, tot)) xr_update(sl[threadIdx.x], P, tot[0], tot[1]);
}

// ---- 32-slot FP32 row kernels, four slots per thread.  Thread tid owns slots
// 4q .. 4q+3 (q = tid & 7) of rows tid / 8 + 32 b + ..., so a row of a [D][32]
// vector is one 128-byte request of eight threads and each thread issues one
// 16-byte load per vector and row: a quarter of the load and index
// instructions of one slot per thread, and the arithmetic on f32x2 pairs.  The
// grid is the one-slot kernels' (row_grid), so the reduction tree is the same.
constexpr int V4_RPB = BS / 8;  // rows per block and step
constexpr int V4_UN = 2;        // rows in flight per thread (L passes; one for six-vector streams)

#define GRID_LOOP4                                                              \
    const int q = threadIdx.x & 7;                                              \
    const int64_t r0i = (int64_t)blockIdx.x * V4_RPB + (threadIdx.x >> 3);      \
    const int64_t rstride = (int64_t)gridDim.x * V4_RPB;
#define ROWS4(Dn, UN) for (int64_t rb = r0i; rb < (Dn); rb += (int64_t)(UN) * rstride)
#define ROWS4_OF_TRIP(rr, UN)                                                   \
    int64_t rr[UN];                                                             \
    _Pragma("unroll") for (int u = 0; u < (UN); ++u) rr[u] = rb + (int64_t)u * rstride;

// bit j set: slot 4q + j is in phase ph
__device__ __forceinline__ unsigned act4(const Slot *sl, int q, int ph) {
    unsigned a = 0;
#pragma unroll
    for (int j = 0; j < 4; ++j) a |= (sl[4 * q + j].phase == ph ? 1u : 0u) << j;
    return a;
}
// all-ones lanes of the active slots, per f32x2 pair
__device__ __forceinline__ void mask4(unsigned a, uint64_t &m0, uint64_t &m1) {
    m0 = ((a & 1u) ? 0xffffffffull : 0ull) | ((a & 2u) ? 0xffffffff00000000ull : 0ull);
    m1 = ((a & 4u) ? 0xffffffffull : 0ull) | ((a & 8u) ? 0xffffffff00000000ull : 0ull);
}
__device__ __forceinline__ ulonglong2 ld4(const float *__restrict__ v, int64_t row, int q) {
    return *(const ulonglong2 *)(v + (uint32_t)row * 32u + 4 * q);
}
// the active slots' values of a row (one 16-byte store when all four are)
__device__ __forceinline__ void st4(float *v, int64_t row, int q, ulonglong2 a, unsigned act) {
    float *p = v + (uint32_t)row * 32u + 4 * q;
    if (act == 15u) {
        *(ulonglong2 *)p = a;
        return;
    }
    float e[4];
    f2_unpack(a.x, e[0], e[1]);
    f2_unpack(a.y, e[2], e[3]);
#pragma unroll
    for (int j = 0; j < 4; ++j)
        if (act & (1u << j)) p[j] = e[j];
}
// per-slot f32x2 pairs of four slots' scalars
__device__ __forceinline__ void slot_pairs(const Slot *sl, int q, double Slot::*f, uint64_t &a0, uint64_t &a1) {
    a0 = f2_pack((float)(sl[4 * q].*f), (float)(sl[4 * q + 1].*f));
    a1 = f2_pack((float)(sl[4 * q + 2].*f), (float)(sl[4 * q + 3].*f));
}

// Dot<float, N> for four slots on f32x2 pairs: exact products p + e, p added
// by TwoSum, errors collected in the low words.  Inactive slots' products are
// masked to zero (their operands are not read for them, and may be anything).
template <int N>
struct Dot4 {
    uint64_t hi[N][2], lo[N][2];
    __device__ __forceinline__ Dot4() {
#pragma unroll
        for (int d = 0; d < N; ++d) hi[d][0] = hi[d][1] = lo[d][0] = lo[d][1] = 0ull;
    }
    __device__ __forceinline__ static void add2(uint64_t &h, uint64_t &l, uint64_t x, uint64_t y, uint64_t msk) {
        const uint64_t p0 = f2_mul(x, y);
        const uint64_t e = f2_fma(x, y, p0 ^ 0x8000000080000000ull) & msk;  // x*y - p0, exactly
        const uint64_t p = p0 & msk;
        const uint64_t s = f2_add(h, p);
        const uint64_t bp = f2_sub(s, h);
        const uint64_t err = f2_add(f2_sub(h, f2_sub(s, bp)), f2_sub(p, bp));
        h = s;
        l = f2_add(l, f2_add(err, e));
    }
    __device__ __forceinline__ void add(int d, ulonglong2 x, ulonglong2 y, uint64_t m0, uint64_t m1) {
        add2(hi[d][0], lo[d][0], x.x, y.x, m0);
        add2(hi[d][1], lo[d][1], x.y, y.y, m1);
    }
};

// double-float sum (a + b): TwoSum of the high words, low words added
__device__ __forceinline__ void df_add(float &h, float &l, float bh, float bl) {
    const float sum = __fadd_rn(h, bh);
    const float bp = __fsub_rn(sum, h);
    const float err = __fadd_rn(__fsub_rn(h, __fsub_rn(sum, bp)), __fsub_rn(bh, bp));
    h = sum;
    l = __fadd_rn(l, __fadd_rn(bl, err));
}

// the block's per-slot sums in double-float on the FP32 pipes (lanes with
// equal q by shuffles, then the eight warps by the first 32 threads), one
// conversion to FP64 per slot and dot, then the grid reduction
template <int N>
__device__ __forceinline__ bool grid_reduce4(const Dot4<N> &acc, double *partial, unsigned int *counter, double (&out)[N]) {
    __shared__ float red[N][2][BS / 32][32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    float h[N][4], l[N][4];
#pragma unroll
    for (int d = 0; d < N; ++d)
#pragma unroll
        for (int p = 0; p < 2; ++p) {
            f2_unpack(acc.hi[d][p], h[d][2 * p], h[d][2 * p + 1]);
            f2_unpack(acc.lo[d][p], l[d][2 * p], l[d][2 * p + 1]);
        }
#pragma unroll
    for (int o = 8; o <= 16; o <<= 1)
#pragma unroll
        for (int d = 0; d < N; ++d)
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const float bh = __shfl_xor_sync(FULL, h[d][j], o), bl = __shfl_xor_sync(FULL, l[d][j], o);
                df_add(h[d][j], l[d][j], bh, bl);
            }
    if (lane < 8)
#pragma unroll
        for (int d = 0; d < N; ++d)
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                red[d][0][warp][4 * lane + j] = h[d][j];
                red[d][1][warp][4 * lane + j] = l[d][j];
            }
    __syncthreads();
    double v[N];
    if (threadIdx.x < 32)
#pragma unroll
        for (int d = 0; d < N; ++d) {
            float sh = red[d][0][0][lane], sl = red[d][1][0][lane];
#pragma unroll
            for (int w = 1; w < BS / 32; ++w) df_add(sh, sl, red[d][0][w][lane], red[d][1][w][lane]);
            v[d] = (double)sh + (double)sl;
        }
    return grid_reduce<32, N, true>(v, partial, counter, out);
}

// k_lpass for 32 FP32 slots (every slot); OVL as in l_rows4
template <bool OVL>
__global__ void __launch_bounds__(BS, 4) k_lpass4(OpView<float> op, float m, float n, const float *__restrict__ x,
                                               const float *__restrict__ t, float *__restrict__ y) {
    GRID_LOOP4
    ROWS4(op.D, V4_UN) {
        ROWS4_OF_TRIP(rr, V4_UN)
        ulonglong2 v[V4_UN];
        l_rows4<V4_UN, OVL>(op, rr, q, m, n, x, t, v);
#pragma unroll
        for (int u = 0; u < V4_UN; ++u)
            if (rr[u] < op.D) st4(y, rr[u], q, v[u], 15u);
    }
}

// the four-slot row kernels read and write 16-byte vectors: caller-owned
// arrays must be 16-byte aligned, and row offsets D * 32 must fit 32 bits
static inline bool lpass4_ok(int64_t D, const void *a, const void *b, const void *c) {
    return D * 32 <= (int64_t)UINT32_MAX && ((uintptr_t)a % 16) == 0 && ((uintptr_t)b % 16) == 0 && ((uintptr_t)c % 16) == 0;
}

// k_apply_alpha for 32 FP32 slots
template <bool OVL>
__global__ void __launch_bounds__(BS, 4) k_apply_alpha4(OpView<float> op, Slot *sl, float m, float n, const float *__restrict__ y,
                                                     const float *__restrict__ te, const float *__restrict__ r0,
                                                     float *__restrict__ v, double *partial, unsigned int *counter) {
    GRID_LOOP4
    const unsigned act = act4(sl, q, PH_ITER);
    uint64_t m0, m1;
    mask4(act, m0, m1);
    Dot4<1> acc;
    if (act)
        ROWS4(op.D, V4_UN) {
            ROWS4_OF_TRIP(rr, V4_UN)
            ulonglong2 r0v[V4_UN], vv[V4_UN];
#pragma unroll
            for (int u = 0; u < V4_UN; ++u) r0v[u] = rr[u] < op.D ? ld4(r0, rr[u], q) : make_ulonglong2(0ull, 0ull);
            l_rows4<V4_UN, OVL>(op, rr, q, m, n, y, te, vv);
#pragma unroll
            for (int u = 0; u < V4_UN; ++u)
                if (rr[u] < op.D) {
                    st4(v, rr[u], q, vv[u], act);
                    acc.add(0, r0v[u], vv[u], m0, m1);
                }
        }
    double tot[1];
    if (grid_reduce4<1>(acc, partial, counter, tot)) alpha_update<float>(sl[threadIdx.x], tot[0]);
}

// k_apply_omega for 32 FP32 slots
template <bool OVL>
__global__ void __launch_bounds__(BS, 4) k_apply_omega4(OpView<float> op, Slot *sl, float m, float n, const float *__restrict__ z,
                                                     const float *__restrict__ te, const float *__restrict__ sv,
                                                     float *__restrict__ tv, double *partial, unsigned int *counter) {
    GRID_LOOP4
    const unsigned act = act4(sl, q, PH_ITER);
    uint64_t m0, m1;
    mask4(act, m0, m1);
    Dot4<2> acc;
    if (act)
        ROWS4(op.D, V4_UN) {
            ROWS4_OF_TRIP(rr, V4_UN)
            ulonglong2 svv[V4_UN], tt[V4_UN];
#pragma unroll
            for (int u = 0; u < V4_UN; ++u) svv[u] = rr[u] < op.D ? ld4(sv, rr[u], q) : make_ulonglong2(0ull, 0ull);
            l_rows4<V4_UN, OVL>(op, rr, q, m, n, z, te, tt);
#pragma unroll
            for (int u = 0; u < V4_UN; ++u)
                if (rr[u] < op.D) {
                    st4(tv, rr[u], q, tt[u], act);
                    acc.add(0, tt[u], tt[u], m0, m1);
                    acc.add(1, tt[u], svv[u], m0, m1);
                }
        }
    double tot[2];
    if (grid_reduce4<2>(acc, partial, counter, tot)) omega_update(sl[threadIdx.x], tot[0], tot[1]);
}

// k_update_xr for 32 FP32 slots
__global__ void __launch_bounds__(BS, 4) k_update_xr4(int64_t D, Slot *sl, SolveParams P, const float *__restrict__ y,
                                                   const float *__restrict__ z, const float *__restrict__ sv,
                                                   const float *__restrict__ tv, const float *__restrict__ r0, float *x,
                                                   float *__restrict__ r, double *partial, unsigned int *counter) {
    GRID_LOOP4
    const unsigned act = act4(sl, q, PH_ITER);
    uint64_t m0, m1;
    mask4(act, m0, m1);
    Dot4<2> acc;
    if (act) {
        uint64_t a0, a1, w0, w1;
        slot_pairs(sl, q, &Slot::alpha, a0, a1);
        slot_pairs(sl, q, &Slot::omega, w0, w1);
        const uint64_t nw0 = w0 ^ 0x8000000080000000ull, nw1 = w1 ^ 0x8000000080000000ull;
        ROWS4(D, 1) {
            ROWS4_OF_TRIP(rr, 1)
            ulonglong2 yv[1], zv[1], xv[1], tw[1], sw[1], r0v[1];
#pragma unroll
            for (int u = 0; u < 1; ++u)
                if (rr[u] < D) {
                    yv[u] = ld4(y, rr[u], q);
                    zv[u] = ld4(z, rr[u], q);
                    xv[u] = *(const ulonglong2 *)(x + (uint32_t)rr[u] * 32u + 4 * q);
                    tw[u] = ld4(tv, rr[u], q);
                    sw[u] = ld4(sv, rr[u], q);
                    r0v[u] = ld4(r0, rr[u], q);
                }
#pragma unroll
            for (int u = 0; u < 1; ++u)
                if (rr[u] < D) {
                    ulonglong2 xn, rn;
                    xn.x = f2_fma(w0, zv[u].x, f2_fma(a0, yv[u].x, xv[u].x));
                    xn.y = f2_fma(w1, zv[u].y, f2_fma(a1, yv[u].y, xv[u].y));
                    rn.x = f2_fma(nw0, tw[u].x, sw[u].x);
                    rn.y = f2_fma(nw1, tw[u].y, sw[u].y);
                    st4(x, rr[u], q, xn, act);
                    st4(r, rr[u], q, rn, act);
                    acc.add(0, rn, rn, m0, m1);
                    acc.add(1, r0v[u], rn, m0, m1);
                }
        }
    }
    double tot[2];
    if (grid_reduce4<2>(acc, partial, counter, tot)) xr_update(sl[threadIdx.x], P, tot[0], tot[1]);
}

// plain-path restart: r = b - A x ; r0 = r ; rho = r0norm2 = ||r||^2
template <class T, int K>
__global__ void __launch_bounds__(BS, 4) k_restart(OpView<T> op, Slot *sl, T m, T n, const double *__restrict__ b,
                                                const T *__restrict__ x, const T *__restrict__ te, T *__restrict__ r,
                                                T *__restrict__ r0, double *partial, unsigned int *counter) {
    GRID_LOOP
    const bool act = sl[s].phase == PH_RESTART;
    Dot<T, 1> acc;
    if (act)
        ROWS_UNR(op.D) {
            ROWS_OF_TRIP(rr)
            double bv[UNR];
            T ax[UNR];
#pragma unroll
            for (int u = 0; u < UNR; ++u) bv[u] = rr[u] < op.D ? b[rr[u] * K + s] : 0.0;
            l_rows<T, K, UNR>(op, rr, s, m, n, x, te, true, ax);
#pragma unroll
            for (int u = 0; u < UNR; ++u)
                if (rr[u] < op.D) {
                    const int64_t i = rr[u] * K + s;
                    T ri = (T)bv[u] - ax[u];
                    r[i] = ri;
                    r0[i] = ri;
                    acc.add(0, ri, ri);
                }
        }
    double av[1], tot[1];
    acc.get(av);
    if (grid_reduce<K, 1>(av, partial, counter, tot)) {
        Slot &S = sl[threadIdx.x];
        if (S.phase != PH_RESTART) return;
        S.rho = S.r0norm2 = tot[0];
        if (S.restarts++ == 0) S.iters = 0;
        S.beta = (S.rho / S.rho_old) * (S.alpha / S.omega);
        S.phase = PH_ITER;
    }
}

// reliable updates run for all slots at once every few iterations, so one FP64
// apply serves every slot that needs it: a slot joins when its FP32 residual has
// fallen by delta since its last update (Sleijpen & van der Vorst's criterion),
// or after four periods without one (an FP32 residual stuck above delta would
// otherwise never meet the true residual, nor the stagnation exit)
template <int K>
__global__ void k_refine_gate(Slot *sl, SolveParams P) {
    const int s = threadIdx.x;
    if (s >= K) return;
    Slot &S = sl[s];
    if (S.phase == PH_ITER && (S.rr <= P.delta * P.delta * S.rr_max || S.upd_iters >= 4 * P.refine_every))
        S.phase = PH_REFINE;
}

// reliable update, step 1: x64 += scale * u32, u32 = 0
template <int K>
__global__ void k_refine_accumulate(int64_t D, const Slot *__restrict__ sl, float *__restrict__ u, double *__restrict__ x64) {
    int64_t gid = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    int64_t row = gid / K;
    int s = (int)(gid % K);
    if (row >= D || sl[s].phase != PH_REFINE) return;
    x64[row * K + s] += sl[s].scale * (double)u[row * K + s];
    u[row * K + s] = 0.0f;
}

// step 2: r64 = b - A x64 (FP64) and ||r64||: done, or replace the FP32 residual
template <int K>
__global__ void __launch_bounds__(BS, 4) k_refine_residual(OpView<double> op, Slot *sl, SolveParams P, double m, double n,
                                                        const double *__restrict__ b, const double *__restrict__ x64,
                                                        const double *__restrict__ te, double *__restrict__ r64,
                                                        double *partial, unsigned int *counter) {
    GRID_LOOP
    const bool act = sl[s].phase == PH_REFINE;
    double acc[1] = {0.0};
    if (act)
        ROWS_UNR(op.D) {
            ROWS_OF_TRIP(rr)
            double bv[UNR], ax[UNR];
#pragma unroll
            for (int u = 0; u < UNR; ++u) bv[u] = rr[u] < op.D ? b[rr[u] * K + s] : 0.0;
            l_rows<double, K, UNR>(op, rr, s, m, n, x64, te, true, ax);
#pragma unroll
            for (int u = 0; u < UNR; ++u)
                if (rr[u] < op.D) {
                    const double ri = bv[u] - ax[u];
                    r64[rr[u] * K + s] = ri;
                    acc[0] += ri * ri;
                }
        }
    double tot[1];
    if (grid_reduce<K, 1>(acc, partial, counter, tot)) {
        Slot &S = sl[threadIdx.x];
        if (S.phase != PH_REFINE) return;
        S.refinements += 1;
        S.rnorm64 = sqrt(tot[0]);
        if (S.rnorm64 < 0.9 * S.rbest) {
            S.rbest = S.rnorm64;
            S.stall = 0;
        } else {
            S.stall += 1;
        }
        if (tot[0] <= S.outer_tol2) {
            S.phase = PH_DONE;
            S.status = 0;
        } else if (S.refinements >= P.max_refine || S.iters >= P.max_iters || !isfinite(tot[0]) || S.stall >= 16 ||
                   S.rnorm64 > 1e6 * sqrt(S.b64norm2)) {
            // out of budget, non-finite, no 10% gain of the true residual in 16
            // reliable updates, or diverged: the FP32 iteration cannot solve this system
            S.phase = PH_DONE;
            S.status = isfinite(tot[0]) ? CPM_ERR_NOT_CONVERGED : CPM_ERR_BREAKDOWN;
        } else {
            S.phase = PH_RELIABLE;
        }
    }
}

// step 3: r32 = r64 / scale; keep p, v, r0 and the scalars, recompute rho = r0 . r
// (after a rho breakdown the Krylov space restarts from the true residual instead)
template <int K>
__global__ void __launch_bounds__(BS, 4) k_reliable(int64_t D, Slot *sl, const double *__restrict__ r64, float *__restrict__ r,
                                                 float *__restrict__ r0, float *__restrict__ p, float *__restrict__ v,
                                                 double *partial, unsigned int *counter) {
    GRID_LOOP
    const bool act = sl[s].phase == PH_RELIABLE;
    const bool fresh = act && sl[s].krylov_restart;
    Dot<float, 2> acc;
    if (act) {
        const double inv = 1.0 / sl[s].scale;
        ROWS_UNR(D) {
            ROWS_OF_TRIP(rr)
            double rv[UNR];
            float r0v[UNR];
#pragma unroll
            for (int u = 0; u < UNR; ++u)
                if (rr[u] < D) {
                    rv[u] = r64[rr[u] * K + s];
                    r0v[u] = fresh ? 0.0f : r0[rr[u] * K + s];
                }
#pragma unroll
            for (int u = 0; u < UNR; ++u)
                if (rr[u] < D) {
                    const int64_t i = rr[u] * K + s;
                    float ri = (float)(rv[u] * inv);
                    r[i] = ri;
                    if (fresh) {
                        r0[i] = ri;
                        p[i] = 0.0f;
                        v[i] = 0.0f;
                    }
                    acc.add(0, ri, ri);
                    acc.add(1, fresh ? ri : r0v[u], ri);
                }
        }
    }
    double av[2], tot[2];
    acc.get(av);
    if (grid_reduce<K, 2>(av, partial, counter, tot)) {
        Slot &S = sl[threadIdx.x];
        if (S.phase != PH_RELIABLE) return;
        S.rr = tot[0];
        S.rr_max = tot[0];
        S.rr_upd = tot[0];
        S.upd_iters = 0;
        if (S.krylov_restart) {
            S.krylov_restart = 0;
            S.restarts += 1;
            S.r0norm2 = tot[0];
            S.rho_old = 1.0;
            S.alpha = 1.0;
            S.omega = 1.0;
        }
        S.rho = tot[1];
        S.beta = (S.rho / S.rho_old) * (S.alpha / S.omega);
        S.phase = PH_ITER;
    }
}

// mixed-path start of the slots in PH_START: x64 = 0, r64 = b, ||b||
template <int K>
__global__ void __launch_bounds__(BS, 4) k_mixed_start(int64_t D, Slot *sl, SolveParams P, const double *__restrict__ b,
                                                    double *__restrict__ x64, double *__restrict__ r64, double *partial,
                                                    unsigned int *counter) {
    GRID_LOOP
    const bool act = sl[s].phase == PH_START;
    double acc[1] = {0.0};
    if (act)
        ROWS_UNR(D) {
            ROWS_OF_TRIP(rr)
            double bv[UNR];
#pragma unroll
            for (int u = 0; u < UNR; ++u) bv[u] = rr[u] < D ? b[rr[u] * K + s] : 0.0;
#pragma unroll
            for (int u = 0; u < UNR; ++u)
                if (rr[u] < D) {
                    const int64_t i = rr[u] * K + s;
                    x64[i] = 0.0;
                    r64[i] = bv[u];
                    acc[0] += bv[u] * bv[u];
                }
        }
    double tot[1];
    if (grid_reduce<K, 1>(acc, partial, counter, tot)) {
        Slot &S = sl[threadIdx.x];
        if (S.phase != PH_START) return;
        S.b64norm2 = tot[0];
        S.outer_tol2 = P.tol * P.tol * tot[0];
        S.iters = 0;
        S.refinements = 0;
        S.restarts = 0;
        S.rnorm64 = sqrt(tot[0]);
        if (!isfinite(tot[0])) {
            S.phase = PH_DONE;
            S.status = CPM_ERR_BREAKDOWN;
            return;
        }
        if (tot[0] == 0.0) {
            S.phase = PH_DONE;
            S.status = 0;
            return;
        }
        S.scale = S.rnorm64;
        S.rbest = S.rnorm64;
        S.stall = 0;
        S.phase = PH_INNER_INIT;
    }
}

// D^-1 denominators m + n L_rr (src/GeneralizedBiCGStabSystem.h:281-340); identity rows 1
template <class T>
__global__ void k_pden(OpView<T> op, double m, double n, T *__restrict__ pden) {
    int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (r >= op.D) return;
    if (op.flags[r] & F_IDENT) {
        pden[r] = (T)1;
        return;
    }
    double ld = (r < op.N) ? (double)op.Ldiag : (double)op.ldiag[r - op.N];
    pden[r] = (T)(m + ld * n);
}

// one slot column of a [D][K] array from / to a contiguous vector
__global__ void k_scatter_col(int64_t D, int K, int j, const double *__restrict__ src, double *__restrict__ dst) {
    int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (r < D) dst[r * K + j] = src[r];
}
__global__ void k_gather_col(int64_t D, int K, int j, const double *__restrict__ src, double *__restrict__ dst) {
    int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (r < D) dst[r] = src[r * K + j];
}

// layout transposes between RHS-major host arrays and [D][K] slot layout
__global__ void k_scatter_cols(int64_t D, int K, int k, const double *__restrict__ src, double *__restrict__ dst) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= D * K) return;
    int64_t row = i / K;
    int s = (int)(i % K);
    dst[i] = (s < k) ? src[(int64_t)s * D + row] : 0.0;
}
__global__ void k_gather_cols(int64_t D, int K, int k, const double *__restrict__ src, double *__restrict__ dst) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= D * (int64_t)k) return;
    int s = (int)(i / D);
    int64_t row = i % D;
    dst[i] = src[row * K + s];
}

}  // namespace cpm

using namespace cpm;

// ================================================================= solver object

struct cpm_solver_s {
    cpm_opset_s *op = nullptr;
    double m = 0, n = 0;
    int K = 1;
    int64_t D = 0;
    int G = 1;
    DBuf<Slot> slots;
    PinnedArray<Slot> h_slots;  // pinned: the slot read-back after a graph does not block the host
    DBuf<double> partial;
    DBuf<unsigned int> counter;
    // FP64 Krylov vectors (plain path) and FP64 refinement state (mixed path)
    DBuf<double> b64, x64, r64, te64, pden64;
    DBuf<double> dr, dr0, dp, dv, ds, dt, dy, dz;
    // FP32 Krylov vectors of the mixed path
    DBuf<float> fx, fr, fr0, fp, fv, fs, ft, fy, fz, fte, pden32;
    bool have64 = false, have32 = false;
    // captured iteration graphs (kernel arguments are fixed pointers; per-solve
    // parameters live in device memory, so a graph is reused while they match)
    cudaGraphExec_t g_plain = nullptr, g_mixed = nullptr;
    SolveParams gp_plain{}, gp_mixed{};
    int chunk = 16;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    cpm_solver_s *fb1 = nullptr;  // 32 slots: one-slot FP64 solver for a few mixed solves to redo
    // the solver's own stream: its work is ordered after the caller's stream at every
    // entry, and two solvers (of one server, say) run concurrently
    cudaStream_t own = nullptr;
    cudaEvent_t entry = nullptr;
    ~cpm_solver_s() {
        if (own) cudaStreamSynchronize(own);
        if (g_plain) cudaGraphExecDestroy(g_plain);
        if (g_mixed) cudaGraphExecDestroy(g_mixed);
        if (e0) cudaEventDestroy(e0);
        if (e1) cudaEventDestroy(e1);
        if (entry) cudaEventDestroy(entry);
        delete fb1;
        if (own) cudaStreamDestroy(own);
    }
};

namespace cpm {
// a solver entry point's work on the solver's stream, ordered after the work the
// calling thread has already queued on its current stream
struct SolverScope {
    StreamScope scope;
    explicit SolverScope(cpm_solver_s *s) : scope(enter(s)) {}
    static cudaStream_t enter(cpm_solver_s *s) {
        cudaEventRecord(s->entry, stream());
        cudaStreamWaitEvent(s->own, s->entry, 0);
        return s->own;
    }
};
}  // namespace cpm

namespace cpm {

static inline unsigned nblk(int64_t n) { return (unsigned)((n + BS - 1) / BS); }

// Jacobi sweeps 2..n of the preconditioner on A y = c (sweep 1 is fused into
// k_update_p / k_update_s)
template <int K>
static void jacobi_rest(cpm_solver_s *s, const SolveParams &P, const double *c, double *y) {
    auto op = s->op->view<double>();
    cudaStream_t st = stream();
    for (int j = 1; j < P.sweeps; ++j) {
        launch_epass<double, K>(op, s->slots.p, PH_ITER, y, s->te64.p, st);
        k_jacobi_sweep<double, K><<<s->G, BS, 0, st>>>(op, s->slots.p, s->m, s->n, c, s->te64.p, s->pden64.p, JACOBI_OMEGA, y);
    }
}

template <int K>
static void plain_iteration(cpm_solver_s *s, const SolveParams &P) {
    auto op = s->op->view<double>();
    const int64_t D = s->D;
    cudaStream_t st = stream();
    Slot *sl = s->slots.p;
    const double *pden = P.precond == 0 ? nullptr : s->pden64.p;
    const double ys = P.precond == 2 ? JACOBI_OMEGA : 1.0;
    k_update_p<double, K><<<s->G, BS, 0, st>>>(D, sl, pden, ys, s->dr.p, s->dv.p, s->dp.p, s->dy.p, s->dr0.p);
    if (P.precond == 2) jacobi_rest<K>(s, P, s->dp.p, s->dy.p);
    launch_epass<double, K>(op, sl, PH_ITER, s->dy.p, s->te64.p, st);
    k_apply_alpha<double, K><<<s->G, BS, 0, st>>>(op, sl, s->m, s->n, s->dy.p, s->te64.p, s->dr0.p, s->dv.p, s->partial.p,
                                                  s->counter.p);
    k_update_s<double, K><<<s->G, BS, 0, st>>>(D, sl, pden, ys, s->dr.p, s->dv.p, s->ds.p, s->dz.p);
    if (P.precond == 2) jacobi_rest<K>(s, P, s->ds.p, s->dz.p);
    launch_epass<double, K>(op, sl, PH_ITER, s->dz.p, s->te64.p, st);
    k_apply_omega<double, K><<<s->G, BS, 0, st>>>(op, sl, s->m, s->n, s->dz.p, s->te64.p, s->ds.p, s->dt.p, s->partial.p,
                                                  s->counter.p);
    k_update_xr<double, K><<<s->G, BS, 0, st>>>(D, sl, P, s->dy.p, s->dz.p, s->ds.p, s->dt.p, s->dr0.p, s->x64.p, s->dr.p,
                                                s->partial.p, s->counter.p);
}

template <int K>
static void plain_restart(cpm_solver_s *s) {
    auto op = s->op->view<double>();
    cudaStream_t st = stream();
    launch_epass<double, K>(op, s->slots.p, PH_RESTART, s->x64.p, s->te64.p, st);
    k_restart<double, K><<<s->G, BS, 0, st>>>(op, s->slots.p, s->m, s->n, s->b64.p, s->x64.p, s->te64.p, s->dr.p, s->dr0.p,
                                              s->partial.p, s->counter.p);
}

template <int K>
static void mixed_iteration(cpm_solver_s *s, const SolveParams &P) {
    auto op = s->op->view<float>();
    const int64_t D = s->D;
    cudaStream_t st = stream();
    Slot *sl = s->slots.p;
    const float m = (float)s->m, n = (float)s->n;
    const float *pden = P.precond == 0 ? nullptr : s->pden32.p;
    // four slots per thread: 32 slots, and row offsets D * 32 within 32 bits
    const bool v4 = (K == 32) && D * 32 <= (int64_t)UINT32_MAX;
    k_update_p<float, K><<<s->G, BS, 0, st>>>(D, sl, pden, 1.0f, s->fr.p, s->fv.p, s->fp.p, s->fy.p, s->fr0.p);
    launch_epass<float, K>(op, sl, PH_ITER, s->fy.p, s->fte.p, st);
    if (v4)
        if (op.ov_ptr)
            k_apply_alpha4<true><<<s->G, BS, 0, st>>>(op, sl, m, n, s->fy.p, s->fte.p, s->fr0.p, s->fv.p, s->partial.p, s->counter.p);
        else
            k_apply_alpha4<false><<<s->G, BS, 0, st>>>(op, sl, m, n, s->fy.p, s->fte.p, s->fr0.p, s->fv.p, s->partial.p, s->counter.p);
    else
        k_apply_alpha<float, K><<<s->G, BS, 0, st>>>(op, sl, m, n, s->fy.p, s->fte.p, s->fr0.p, s->fv.p, s->partial.p,
                                                     s->counter.p);
    k_update_s<float, K><<<s->G, BS, 0, st>>>(D, sl, pden, 1.0f, s->fr.p, s->fv.p, s->fs.p, s->fz.p);
    launch_epass<float, K>(op, sl, PH_ITER, s->fz.p, s->fte.p, st);
    if (v4) {
        if (op.ov_ptr)
            k_apply_omega4<true><<<s->G, BS, 0, st>>>(op, sl, m, n, s->fz.p, s->fte.p, s->fs.p, s->ft.p, s->partial.p, s->counter.p);
        else
            k_apply_omega4<false><<<s->G, BS, 0, st>>>(op, sl, m, n, s->fz.p, s->fte.p, s->fs.p, s->ft.p, s->partial.p, s->counter.p);
        k_update_xr4<<<s->G, BS, 0, st>>>(D, sl, P, s->fy.p, s->fz.p, s->fs.p, s->ft.p, s->fr0.p, s->fx.p, s->fr.p,
                                          s->partial.p, s->counter.p);
    } else {
        k_apply_omega<float, K><<<s->G, BS, 0, st>>>(op, sl, m, n, s->fz.p, s->fte.p, s->fs.p, s->ft.p, s->partial.p,
                                                     s->counter.p);
        k_update_xr<float, K><<<s->G, BS, 0, st>>>(D, sl, P, s->fy.p, s->fz.p, s->fs.p, s->ft.p, s->fr0.p, s->fx.p, s->fr.p,
                                                   s->partial.p, s->counter.p);
    }
}

// reliable update (FP64) for slots that asked for one
template <int K>
static void mixed_refine(cpm_solver_s *s, const SolveParams &P) {
    auto op64 = s->op->view<double>();
    const int64_t D = s->D;
    cudaStream_t st = stream();
    Slot *sl = s->slots.p;
    k_refine_gate<K><<<1, 32, 0, st>>>(sl, P);
    k_refine_accumulate<K><<<nblk(D * K), BS, 0, st>>>(D, sl, s->fx.p, s->x64.p);
    launch_epass<double, K>(op64, sl, PH_REFINE, s->x64.p, s->te64.p, st);
    k_refine_residual<K><<<s->G, BS, 0, st>>>(op64, sl, P, s->m, s->n, s->b64.p, s->x64.p, s->te64.p, s->r64.p, s->partial.p,
                                              s->counter.p);
    k_reliable<K><<<s->G, BS, 0, st>>>(D, sl, s->r64.p, s->fr.p, s->fr0.p, s->fp.p, s->fv.p, s->partial.p, s->counter.p);
}

static int alloc_vectors(cpm_solver_s *s, bool want64, bool want32) {
    const size_t n = (size_t)s->D * s->K;
    if (want64 && !s->have64) {
        for (auto *b : {&s->dr, &s->dr0, &s->dp, &s->dv, &s->ds, &s->dt, &s->dy, &s->dz}) CPM_TRY(b->alloc(n));
        s->have64 = true;
    }
    if (want32 && !s->have32) {
        for (auto *b : {&s->fx, &s->fr, &s->fr0, &s->fp, &s->fv, &s->fs, &s->ft, &s->fy, &s->fz, &s->fte}) CPM_TRY(b->alloc(n));
        CPM_TRY(s->pden32.alloc(s->D));
        k_pden<float><<<nblk(s->D), BS, 0, stream()>>>(s->op->view<float>(), s->m, s->n, s->pden32.p);
        CPM_CUDA_TRY(cudaGetLastError());
        s->have32 = true;
    }
    return 0;
}

static bool same_params(const SolveParams &a, const SolveParams &b) {
    return a.tol == b.tol && a.delta == b.delta && a.max_iters == b.max_iters && a.max_refine == b.max_refine &&
           a.mixed == b.mixed && a.precond == b.precond && a.sweeps == b.sweeps && a.refine_every == b.refine_every;
}


static int parse_params(const cpm_solve_opts *o, SolveParams &P) {
    memset(&P, 0, sizeof(P));
    P.tol = o->tol > 0 ? o->tol : 1e-10;
    P.max_iters = o->max_iters > 0 ? o->max_iters : 100000;
    P.mixed = o->precision == 1;
    P.delta = o->inner_tol > 0 ? o->inner_tol : 0.1;
    P.max_refine = o->max_refine > 0 ? o->max_refine : 400;
    P.refine_every = o->refine_every > 0 ? o->refine_every : 32;
    if (P.refine_every > 32 || (P.refine_every & (P.refine_every - 1)))
        return fail(CPM_ERR_INVALID_ARG, "refine_every must be 1, 2, 4, 8, 16 or 32");
    P.precond = o->precond;
    P.sweeps = o->precond_iters;
    if (P.precond < 0 || P.precond > 2) return fail(CPM_ERR_INVALID_ARG, "precond must be 0 (identity), 1 (diagonal) or 2 (jacobi)");
    if (P.precond == 2 && (P.sweeps < 1 || P.sweeps > 20000))
        return fail(CPM_ERR_INVALID_ARG, "the jacobi preconditioner needs 1 <= precond_iters <= 20000");
    // FP32 cannot hold the far-field values that many Jacobi sweeps resolve (a
    // heat kernel decays below 1e-38 within a few hundred cells), so the Jacobi
    // preconditioner is an FP64 solve
    if (P.precond == 2 && P.mixed)
        return fail(CPM_ERR_UNSUPPORTED, "the jacobi preconditioner runs in FP64 (precision 0) only");
    return 0;
}

// iterations per captured graph
// (Jacobi-preconditioned solves: one iteration, already thousands of launches;
// mixed: 32 iterations, so that the reliable-update period can reach 32)
static inline int graph_chunk(const cpm_solver_s *s, const SolveParams &P) {
    return (P.precond == 2) ? 1 : (P.mixed ? 2 * s->chunk : s->chunk);
}

// the captured iteration graph for P (reused while the parameters match)
template <int K>
static int prepare_graph(cpm_solver_s *s, const SolveParams &P, cudaGraphExec_t *out) {
    cudaStream_t st = stream();
    cudaGraphExec_t &gexec = P.mixed ? s->g_mixed : s->g_plain;
    SolveParams &gpar = P.mixed ? s->gp_mixed : s->gp_plain;
    if (gexec && !same_params(gpar, P)) {
        cudaGraphExecDestroy(gexec);
        gexec = nullptr;
    }
    if (!gexec) {
        cudaGraph_t graph;
        CPM_CUDA_TRY(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
        const int chunk = graph_chunk(s, P);
        for (int it = 0; it < chunk; ++it) {
            if (P.mixed) {
                mixed_iteration<K>(s, P);
                if (it % P.refine_every == P.refine_every - 1) mixed_refine<K>(s, P);
            } else {
                plain_iteration<K>(s, P);
            }
        }
        cudaError_t ce = cudaStreamEndCapture(st, &graph);
        if (ce != cudaSuccess) return fail(CPM_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(ce));
        ce = cudaGraphInstantiate(&gexec, graph, 0);
        cudaGraphDestroy(graph);
        if (ce != cudaSuccess) return fail(CPM_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(ce));
        gpar = P;
    }
    *out = gexec;
    return 0;
}

// kernels launched by one graph replay
static inline long long graph_launches(const cpm_solver_s *s, const SolveParams &P) {
    const int chunk = graph_chunk(s, P);
    // an iteration: 5 vector / L-pass kernels and two E passes; a Jacobi sweep: an E
    // pass and the sweep; a reliable update: 4 kernels and an FP64 E pass
    const long long e32 = s->K == 32 ? epass_kernels<float, 32>(s->op->view<float>(), s->fy.p) : 1;
    const long long e64 = s->K == 32 ? epass_kernels<double, 32>(s->op->view<double>(), s->x64.p) : 1;
    const long long eit = P.mixed ? e32 : e64;
    return (5LL + 2 * eit + (P.precond == 2 ? 2LL * (P.sweeps - 1) * (e64 + 1) : 0)) * chunk +
           (P.mixed ? (4LL + e64) * (chunk / P.refine_every) : 0);
}

// start the mixed-path slots in PH_START (FP64 residual, then the FP32 Krylov state)
template <int K>
static void mixed_start(cpm_solver_s *s, const SolveParams &P) {
    cudaStream_t st = stream();
    k_mixed_start<K><<<s->G, BS, 0, st>>>(s->D, s->slots.p, P, s->b64.p, s->x64.p, s->r64.p, s->partial.p, s->counter.p);
    k_init<float, K><<<s->G, BS, 0, st>>>(s->op->view<float>(), s->slots.p, P, PH_INNER_INIT, s->r64.p, s->fx.p, s->fr.p,
                                          s->fr0.p, s->fp.p, s->fv.p, s->partial.p, s->counter.p);
    count_launches(2);
}

static void slot_stats(const Slot &S, bool mixed, float ms, cpm_solve_stats *st) {
    const int status = (S.phase == PH_DONE) ? S.status : CPM_ERR_TIMEOUT;
    st->iterations = S.iters;
    st->refinements = S.refinements;
    st->restarts = S.restarts;
    st->status = status;
    st->rel_residual = mixed ? (S.b64norm2 > 0 ? S.rnorm64 / std::sqrt(S.b64norm2) : 0.0)
                             : (S.bnorm2 > 0 ? std::sqrt(S.rr / S.bnorm2) : 0.0);
    st->seconds = ms * 1e-3;
    st->fp64_fallback = 0;
    st->pad = 0;
}

// One pass of the slot loop for the slots in `active` (others idle): the
// start kernels, then iteration graphs until every active slot is done.
template <int K>
static int solve_pass(cpm_solver_s *s, const SolveParams &P, const std::vector<char> &active, float *ms) {
    CPM_TRY(alloc_vectors(s, !P.mixed, P.mixed));
    cudaStream_t st = stream();
    for (int j = 0; j < K; ++j) {
        memset(&s->h_slots[j], 0, sizeof(Slot));
        s->h_slots[j].phase = active[j] ? (P.mixed ? PH_START : PH_ITER) : PH_IDLE;
    }
    CPM_CUDA_TRY(cudaMemcpyAsync(s->slots.p, s->h_slots.data(), sizeof(Slot) * K, cudaMemcpyHostToDevice, st));
    CPM_CUDA_TRY(cudaEventRecord(s->e0, st));
    if (!P.mixed) {
        k_init<double, K><<<s->G, BS, 0, st>>>(s->op->view<double>(), s->slots.p, P, PH_ITER, s->b64.p, s->x64.p, s->dr.p,
                                               s->dr0.p, s->dp.p, s->dv.p, s->partial.p, s->counter.p);
        count_launches(1);
    } else {
        mixed_start<K>(s, P);
    }
    CPM_CUDA_TRY(cudaGetLastError());
    cudaGraphExec_t gexec = nullptr;
    CPM_TRY(prepare_graph<K>(s, P, &gexec));
    const int chunk = graph_chunk(s, P);
    const int64_t max_chunks = (int64_t)P.max_iters / chunk + 2 * P.max_refine + 4;
    const long long per_graph = graph_launches(s, P);
    bool done = false;
    for (int64_t c = 0; c < max_chunks && !done; ++c) {
        CPM_CUDA_TRY(cudaGraphLaunch(gexec, st));
        count_launches(per_graph);
        CPM_CUDA_TRY(cudaMemcpyAsync(s->h_slots.data(), s->slots.p, sizeof(Slot) * K, cudaMemcpyDeviceToHost, st));
        CPM_CUDA_TRY(cudaStreamSynchronize(st));
        done = true;
        bool restart = false;
        for (int j = 0; j < K; ++j) {
            int ph = s->h_slots[j].phase;
            if (ph != PH_DONE && ph != PH_IDLE) done = false;
            if (ph == PH_RESTART) restart = true;
        }
        if (restart && !P.mixed) {
            plain_restart<K>(s);
            count_launches(2);
            CPM_CUDA_TRY(cudaGetLastError());
        }
    }
    CPM_CUDA_TRY(cudaEventRecord(s->e1, st));
    CPM_CUDA_TRY(cudaEventSynchronize(s->e1));
    *ms = 0;
    cudaEventElapsedTime(ms, s->e0, s->e1);
    return 0;
}

// Solve k right-hand sides.  A mixed-precision slot that does not converge
// (an FP32 inner iteration that cannot follow an ill-conditioned system, where
// cond * 2^-24 ~ 1) is solved again by the plain FP64 path from x = 0; its
// stats then carry fp64_fallback = 1 and both passes' iterations.
template <int K>
static int run_solve(cpm_solver_s *s, int k, const cpm_solve_opts *o, cpm_solve_stats *stats) {
    SolveParams P;
    CPM_TRY(parse_params(o, P));
    if (P.mixed && s->op->n_sp_rows > 0)
        return fail(CPM_ERR_UNSUPPORTED, "an operator with per-slot patches is solved in FP64 (precision 0)");
    std::vector<char> active(K, 0);
    for (int j = 0; j < k; ++j) active[j] = 1;
    float ms = 0;
    CPM_TRY(solve_pass<K>(s, P, active, &ms));
    std::vector<cpm_solve_stats> st(K);
    std::vector<char> redo(K, 0);
    bool any_redo = false;
    for (int j = 0; j < k; ++j) {
        slot_stats(s->h_slots[j], P.mixed, ms, &st[j]);
        if (P.mixed && st[j].status != 0) redo[j] = any_redo = true;
    }
    int n_redo = 0;
    for (int j = 0; j < k; ++j) n_redo += redo[j];
    // a 32-slot FP64 iteration costs about 14 one-slot ones: a few right-hand sides
    // are solved again one at a time
    if (K == 32 && n_redo > 0 && n_redo < 14) {
        if (!s->fb1) CPM_TRY(cpm_solver_create(s->op, s->m, s->n, 1, &s->fb1));
        cpm_solve_opts o64 = *o;
        o64.precision = 0;
        const int64_t D = s->D;
        for (int j = 0; j < k; ++j) {
            if (!redo[j]) continue;
            k_gather_col<<<nblk(D), BS, 0, stream()>>>(D, 32, j, s->b64.p, s->fb1->b64.p);
            CPM_CUDA_TRY(cudaGetLastError());
            cpm_solve_stats s64;
            const int rc64 = cpm_solve_device(s->fb1, 1, s->fb1->b64.p, nullptr, &o64, &s64);
            if (rc64 != 0 && rc64 != CPM_ERR_NOT_CONVERGED && rc64 != CPM_ERR_BREAKDOWN) return rc64;
            k_scatter_col<<<nblk(D), BS, 0, stream()>>>(D, 32, j, s->fb1->x64.p, s->x64.p);
            CPM_CUDA_TRY(cudaGetLastError());
            s64.iterations += st[j].iterations;
            s64.refinements = st[j].refinements;
            s64.seconds += st[j].seconds;
            s64.fp64_fallback = 1;
            st[j] = s64;
        }
        any_redo = false;
    }
    if (any_redo) {
        SolveParams P64 = P;
        P64.mixed = 0;
        float ms64 = 0;
        CPM_TRY(solve_pass<K>(s, P64, redo, &ms64));
        for (int j = 0; j < k; ++j) {
            if (!redo[j]) {
                st[j].seconds += ms64 * 1e-3;
                continue;
            }
            cpm_solve_stats s64;
            slot_stats(s->h_slots[j], false, ms + ms64, &s64);
            s64.iterations += st[j].iterations;
            s64.refinements = st[j].refinements;
            s64.fp64_fallback = 1;
            st[j] = s64;
        }
    }
    int rc = 0;
    for (int j = 0; j < k; ++j) {
        if (st[j].status != 0 && rc == 0) rc = st[j].status;
        if (stats) stats[j] = st[j];
    }
    if (rc) set_error("solve did not converge for every right-hand side (see per-RHS status)");
    return rc;
}

}  // namespace cpm

extern "C" int cpm_solver_create(cpm_opset_t op, double m, double n, int32_t kslots, cpm_solver_t *out) {
    if (!op || !out || kslots < 1 || kslots > 32) return fail(CPM_ERR_INVALID_ARG, "kslots must be in [1, 32]");
    if (op->n_sp_rows > 0 && kslots != 32)
        return fail(CPM_ERR_UNSUPPORTED, "an operator with per-slot patches is solved with 32 slots");
    *out = nullptr;
    cpm_solver_s *s = new cpm_solver_s();
    if (cudaStreamCreateWithFlags(&s->own, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&s->entry, cudaEventDisableTiming) != cudaSuccess) {
        delete s;
        return fail(CPM_ERR_CUDA, "solver_create: stream");
    }
    SolverScope sc(s);
    s->op = op;
    s->m = m;
    s->n = n;
    s->K = (kslots == 1) ? 1 : 32;
    s->D = op->D;
    s->G = row_grid(s->D, s->K);
    auto bail = [&](int rc) {
        delete s;
        return rc;
    };
    int rc;
    if ((rc = s->h_slots.alloc(s->K)) || (rc = s->slots.alloc(s->K)) || (rc = s->partial.alloc((size_t)(s->G + reduce_groups(s->G)) * s->K * 2)) ||
        (rc = s->counter.alloc((size_t)(1 + reduce_groups(s->G)))) ||
        (rc = s->counter.zero()) || (rc = s->b64.alloc((size_t)s->D * s->K)) || (rc = s->x64.alloc((size_t)s->D * s->K)) ||
        (rc = s->r64.alloc((size_t)s->D * s->K)) || (rc = s->te64.alloc((size_t)s->D * s->K)) || (rc = s->pden64.alloc(s->D)))
        return bail(rc);
    k_pden<double><<<nblk(s->D), BS, 0, stream()>>>(op->view<double>(), m, n, s->pden64.p);
    if (cudaGetLastError() != cudaSuccess) return bail(fail(CPM_ERR_CUDA, "pden kernel"));
    cudaEventCreate(&s->e0);
    cudaEventCreate(&s->e1);
    if (cudaStreamSynchronize(s->own) != cudaSuccess) return bail(fail(CPM_ERR_CUDA, "solver_create"));
    *out = s;
    return 0;
}

extern "C" int cpm_solve_device(cpm_solver_t s, int32_t k, const void *b_dev, void *x_dev, const cpm_solve_opts *opts,
                                cpm_solve_stats *stats) {
    if (!s || !opts || k < 1 || k > s->K) return fail(CPM_ERR_INVALID_ARG, "invalid solve arguments");
    SolverScope sc(s);
    const size_t bytes = (size_t)s->D * s->K * sizeof(double);
    if (b_dev != s->b64.p) CPM_CUDA_TRY(cudaMemcpyAsync(s->b64.p, b_dev, bytes, cudaMemcpyDeviceToDevice, stream()));
    int rc = (s->K == 1) ? run_solve<1>(s, k, opts, stats) : run_solve<32>(s, k, opts, stats);
    if (x_dev) CPM_CUDA_TRY(cudaMemcpyAsync(x_dev, s->x64.p, bytes, cudaMemcpyDeviceToDevice, stream()));
    CPM_CUDA_TRY(cudaStreamSynchronize(stream()));
    return rc;
}

extern "C" int cpm_solve(cpm_solver_t s, int32_t k, const double *b, double *x, const cpm_solve_opts *opts, cpm_solve_stats *stats) {
    if (!s || !b || !x || !opts || k < 1 || k > s->K) return fail(CPM_ERR_INVALID_ARG, "invalid solve arguments");
    SolverScope sc(s);
    DBuf<double> stage;
    CPM_TRY(stage.upload(b, (size_t)s->D * k));
    k_scatter_cols<<<nblk(s->D * s->K), BS, 0, stream()>>>(s->D, s->K, k, stage.p, s->b64.p);
    CPM_CUDA_TRY(cudaGetLastError());
    int rc = (s->K == 1) ? run_solve<1>(s, k, opts, stats) : run_solve<32>(s, k, opts, stats);
    k_gather_cols<<<nblk(s->D * (int64_t)k), BS, 0, stream()>>>(s->D, s->K, k, s->x64.p, stage.p);
    CPM_CUDA_TRY(cudaGetLastError());
    CPM_CUDA_TRY(cudaMemcpyAsync(x, stage.p, sizeof(double) * s->D * k, cudaMemcpyDeviceToHost, stream()));
    CPM_CUDA_TRY(cudaStreamSynchronize(stream()));
    return rc;
}

extern "C" int cpm_solver_destroy(cpm_solver_t s) {
    delete s;
    return 0;
}

// ================================================================= serving
// Continuous batching over the slots of `nb` 32-slot solvers on one operator,
// each on its own stream: a request is admitted into a free slot as soon as one
// frees up (its column of b is written and the slot alone is started, the
// other slots keep their state), every step launches one iteration graph per
// busy solver, all of them queued before any is waited for, so one batch's
// latency-bound E pass overlaps another's bandwidth-bound row kernels; finished
// slots are harvested after the graphs.

struct cpm_server_s {
    std::vector<cpm_solver_s *> solvers;
    cpm_solver_s *fallback = nullptr;  // 1-slot solver for requests the mixed path cannot converge
    SolveParams P{};
    cpm_solve_opts opts{};
    struct Req {
        int64_t tag;
        std::vector<double> b;        // host right-hand side, or
        const double *b_dev = nullptr;  // a device one
        double *x_dev = nullptr;        // device destination of the solution (else host, via poll)
        std::chrono::steady_clock::time_point t_submit;
    };
    struct Busy {
        bool used = false;
        int64_t tag = 0;
        double *x_dev = nullptr;
        std::chrono::steady_clock::time_point t_submit, t_admit;
    };
    struct Done {
        int64_t tag;
        std::vector<double> x;          // the solution, once moved out of the result columns
        const double *pend = nullptr;   // or still in batch pb's pinned result column
        int pb = -1;
        cpm_solve_stats st;
        double latency;
    };
    std::deque<Req> queue;
    std::vector<Busy> busy;     // 32 per solver
    std::deque<Done> done;
    double *h_stage = nullptr;  // pinned, [32 nb][D]: one right-hand-side staging column per slot
    double *h_res = nullptr;    // pinned, [32 nb][D]: one result column per slot
    DBuf<double> d_stage;       // device, [32 nb][D]
    std::vector<char> inflight;         // per batch: launched, not yet harvested
    std::vector<cudaEvent_t> res_ev;    // per batch: its last harvest's copies are done
    ~cpm_server_s() {
        for (auto *s : solvers)
            if (s) cudaStreamSynchronize(s->own);
        if (h_stage) cudaFreeHost(h_stage);
        if (h_res) cudaFreeHost(h_res);
        for (cudaEvent_t e : res_ev)
            if (e) cudaEventDestroy(e);
        for (auto *s : solvers) delete s;
        delete fallback;
    }
};

static int server_create(cpm_opset_t op, double m, double n, const cpm_solve_opts *opts, int nb, cpm_server_t *out) {
    if (!op || !opts || !out) return fail(CPM_ERR_INVALID_ARG, "server_create: null argument");
    *out = nullptr;
    if (nb < 1 || nb > 8) return fail(CPM_ERR_INVALID_ARG, "server_create: 1 to 8 batches");
    if (opts->precision != 0 && opts->precision != 1) return fail(CPM_ERR_INVALID_ARG, "precision must be 0 or 1");
    if (opts->precond != 1) return fail(CPM_ERR_UNSUPPORTED, "the server runs the diagonal preconditioner");
    cpm_server_s *sv = new cpm_server_s();
    auto bail = [&](int rc) {
        delete sv;
        return rc;
    };
    sv->opts = *opts;
    int rc = parse_params(opts, sv->P);
    if (rc) return bail(rc);
    sv->solvers.assign(nb, nullptr);
    for (int b = 0; b < nb && !rc; ++b) rc = cpm_solver_create(op, m, n, 32, &sv->solvers[b]);
    if (rc) return bail(rc);
    const int64_t D = op->D;
    if (cudaMallocHost((void **)&sv->h_stage, sizeof(double) * 32 * nb * (size_t)D) != cudaSuccess ||
        cudaMallocHost((void **)&sv->h_res, sizeof(double) * 32 * nb * (size_t)D) != cudaSuccess)
        return bail(fail(CPM_ERR_OOM, "server_create: pinned staging"));
    sv->inflight.assign(nb, 0);
    sv->res_ev.assign(nb, nullptr);
    for (int b = 0; b < nb; ++b)
        if (cudaEventCreateWithFlags(&sv->res_ev[b], cudaEventDisableTiming) != cudaSuccess)
            return bail(fail(CPM_ERR_CUDA, "server_create: event"));
    if ((rc = sv->d_stage.alloc(32 * nb * (size_t)D))) return bail(rc);
    sv->busy.assign(32 * nb, cpm_server_s::Busy());
    for (cpm_solver_s *s : sv->solvers) {
        SolverScope sc(s);
        if ((rc = alloc_vectors(s, !sv->P.mixed, sv->P.mixed))) return bail(rc);
        for (int j = 0; j < 32; ++j) {
            memset(&s->h_slots[j], 0, sizeof(Slot));
            s->h_slots[j].phase = PH_IDLE;
        }
        CPM_CUDA_TRY(cudaMemcpyAsync(s->slots.p, s->h_slots.data(), sizeof(Slot) * 32, cudaMemcpyHostToDevice, stream()));
        cudaGraphExec_t g = nullptr;
        if ((rc = prepare_graph<32>(s, sv->P, &g))) return bail(rc);
        CPM_CUDA_TRY(cudaStreamSynchronize(stream()));
    }
    *out = sv;
    return 0;
}

extern "C" int cpm_server_create(cpm_opset_t op, double m, double n, const cpm_solve_opts *opts, cpm_server_t *out) {
    return server_create(op, m, n, opts, 1, out);
}

extern "C" int cpm_server_create_batches(cpm_opset_t op, double m, double n, const cpm_solve_opts *opts, int32_t batches,
                                         cpm_server_t *out) {
    return server_create(op, m, n, opts, batches, out);
}

extern "C" int cpm_server_submit(cpm_server_t sv, const double *b, int64_t tag) {
    if (!sv || !b) return fail(CPM_ERR_INVALID_ARG, "server_submit: null argument");
    cpm_server_s::Req r;
    r.tag = tag;
    r.b.assign(b, b + sv->solvers[0]->D);
    r.t_submit = std::chrono::steady_clock::now();
    sv->queue.push_back(std::move(r));
    return 0;
}

extern "C" int cpm_server_submit_device(cpm_server_t sv, const void *b_dev, void *x_dev, int64_t tag) {
    if (!sv || !b_dev || !x_dev) return fail(CPM_ERR_INVALID_ARG, "server_submit_device: null argument");
    cpm_server_s::Req r;
    r.tag = tag;
    r.b_dev = (const double *)b_dev;
    r.x_dev = (double *)x_dev;
    r.t_submit = std::chrono::steady_clock::now();
    sv->queue.push_back(std::move(r));
    return 0;
}

// admit queued requests into batch b's free slots, start them and launch its
// iteration graph (when any slot is busy) and the read-back of its slot states,
// all on the batch's stream without waiting
static int server_launch(cpm_server_t sv, int b) {
    const int64_t D = sv->solvers[0]->D;
    cpm_solver_s *s = sv->solvers[b];
    SolverScope sc(s);
    cudaStream_t st = stream();
    bool admitted = false;
    for (int j = 0; j < 32 && !sv->queue.empty(); ++j) {
        cpm_server_s::Busy &bz = sv->busy[32 * b + j];
        if (bz.used) continue;
        cpm_server_s::Req r = std::move(sv->queue.front());
        sv->queue.pop_front();
        double *hs = sv->h_stage + (size_t)(32 * b + j) * D, *ds = sv->d_stage.p + (size_t)(32 * b + j) * D;
        const double *src = r.b_dev;
        if (!src) {
            memcpy(hs, r.b.data(), sizeof(double) * D);
            CPM_CUDA_TRY(cudaMemcpyAsync(ds, hs, sizeof(double) * D, cudaMemcpyHostToDevice, st));
            src = ds;
        }
        k_scatter_col<<<nblk(D), BS, 0, st>>>(D, 32, j, src, s->b64.p);
        count_launches(1);
        memset(&s->h_slots[j], 0, sizeof(Slot));
        s->h_slots[j].phase = PH_START;
        CPM_CUDA_TRY(cudaMemcpyAsync(s->slots.p + j, &s->h_slots[j], sizeof(Slot), cudaMemcpyHostToDevice, st));
        bz.used = true;
        bz.tag = r.tag;
        bz.x_dev = r.x_dev;
        bz.t_submit = r.t_submit;
        bz.t_admit = std::chrono::steady_clock::now();
        admitted = true;
    }
    if (admitted) {
        if (sv->P.mixed) {
            mixed_start<32>(s, sv->P);
        } else {
            k_init<double, 32><<<s->G, BS, 0, st>>>(s->op->view<double>(), s->slots.p, sv->P, PH_START, s->b64.p, s->x64.p,
                                                    s->dr.p, s->dr0.p, s->dp.p, s->dv.p, s->partial.p, s->counter.p);
            count_launches(1);
        }
    }
    int n_busy = 0;
    for (int j = 0; j < 32; ++j) n_busy += sv->busy[32 * b + j].used;
    if (n_busy) {
        cudaGraphExec_t g = nullptr;
        CPM_TRY(prepare_graph<32>(s, sv->P, &g));
        CPM_CUDA_TRY(cudaGraphLaunch(g, st));
        count_launches(graph_launches(s, sv->P));
    }
    CPM_CUDA_TRY(cudaMemcpyAsync(s->h_slots.data(), s->slots.p, sizeof(Slot) * 32, cudaMemcpyDeviceToHost, st));
    sv->inflight[b] = 1;
    return 0;
}

// wait for batch b's last launch and harvest its finished slots: each solution
// gathered to its device destination, or copied into the batch's pinned result
// columns (poll copies it out once the batch's result event has passed); the
// caller's stream is ordered after the gathers.  Results of the batch still
// unpolled are moved out of those columns first.
static int server_harvest(cpm_server_t sv, int b, cudaStream_t caller, int *n_fin) {
    const int64_t D = sv->solvers[0]->D;
    cpm_solver_s *s = sv->solvers[b];
    SolverScope sc(s);
    cudaStream_t st = stream();
    CPM_CUDA_TRY(cudaStreamSynchronize(st));
    sv->inflight[b] = 0;
    for (cpm_server_s::Done &d : sv->done)
        if (d.pend && d.pb == b) {
            d.x.assign(d.pend, d.pend + D);
            d.pend = nullptr;
        }
    if (!sv->P.mixed) {  // the plain path's restarts run between graphs (as in run_solve)
        bool restart = false;
        for (int j = 0; j < 32; ++j) restart = restart || s->h_slots[j].phase == PH_RESTART;
        if (restart) {
            plain_restart<32>(s);
            count_launches(2);
            CPM_CUDA_TRY(cudaGetLastError());
        }
    }
    std::vector<int> fin;
    std::vector<cpm_solve_stats> fb_st(32);
    std::vector<char> fb(32, 0);
    for (int j = 0; j < 32; ++j) {
        const Slot &S = s->h_slots[j];
        cpm_server_s::Busy &bz = sv->busy[32 * b + j];
        if (!bz.used) continue;
        const bool over = S.phase == PH_DONE || S.iters >= sv->P.max_iters || S.refinements >= sv->P.max_refine;
        if (!over) continue;
        double *ds = bz.x_dev ? bz.x_dev : sv->d_stage.p + (size_t)(32 * b + j) * D;
        if (S.phase == PH_DONE && (S.status == 0 || !sv->P.mixed)) {
            k_gather_col<<<nblk(D), BS, 0, st>>>(D, 32, j, s->x64.p, ds);
            count_launches(1);
        } else {
            // the FP32 inner iteration could not solve this right-hand side:
            // solve it again with the plain FP64 path (one slot, blocking)
            if (!sv->fallback) CPM_TRY(cpm_solver_create(s->op, s->m, s->n, 1, &sv->fallback));
            double *bj = sv->d_stage.p + (size_t)(32 * b + j) * D;
            k_gather_col<<<nblk(D), BS, 0, st>>>(D, 32, j, s->b64.p, bj);
            count_launches(1);
            cpm_solve_opts o64 = sv->opts;
            o64.precision = 0;
            CPM_TRY(cpm_solve_device(sv->fallback, 1, bj, ds, &o64, &fb_st[j]));
            fb[j] = 1;
        }
        if (!bz.x_dev)
            CPM_CUDA_TRY(cudaMemcpyAsync(sv->h_res + (size_t)(32 * b + j) * D, ds, sizeof(double) * D,
                                         cudaMemcpyDeviceToHost, st));
        fin.push_back(j);
    }
    if (fin.empty()) return 0;
    CPM_CUDA_TRY(cudaEventRecord(sv->res_ev[b], st));
    CPM_CUDA_TRY(cudaStreamWaitEvent(caller, sv->res_ev[b], 0));
    const auto now = std::chrono::steady_clock::now();
    for (int j : fin) {
        cpm_server_s::Busy &bz = sv->busy[32 * b + j];
        cpm_server_s::Done d;
        d.tag = bz.tag;
        if (!bz.x_dev) {
            d.pend = sv->h_res + (size_t)(32 * b + j) * D;
            d.pb = b;
        }
        slot_stats(s->h_slots[j], sv->P.mixed != 0, 0.0f, &d.st);
        if (fb[j]) {
            const int it = d.st.iterations, rf = d.st.refinements;
            d.st = fb_st[j];
            d.st.iterations += it;
            d.st.refinements = rf;
            d.st.fp64_fallback = 1;
        }
        d.latency = std::chrono::duration<double>(now - bz.t_submit).count();
        d.st.seconds = std::chrono::duration<double>(now - bz.t_admit).count();
        sv->done.push_back(std::move(d));
        bz.used = false;
        s->h_slots[j].phase = PH_IDLE;
        CPM_CUDA_TRY(cudaMemcpyAsync(s->slots.p + j, &s->h_slots[j], sizeof(Slot), cudaMemcpyHostToDevice, st));
        ++*n_fin;
    }
    return 0;
}

static void server_counts(cpm_server_t sv, int n_fin, int32_t *active, int32_t *queued, int32_t *finished) {
    int n_busy = 0;
    for (auto &bz : sv->busy) n_busy += bz.used;
    if (active) *active = n_busy;
    if (queued) *queued = (int32_t)sv->queue.size();
    if (finished) *finished = n_fin;
}

// One round: admit queued requests into free slots, launch every busy batch's
// iteration graph (each on its own stream, all queued before any is waited for),
// then wait for them and harvest the finished requests.
extern "C" int cpm_server_step(cpm_server_t sv, int32_t *active, int32_t *queued, int32_t *finished) {
    if (!sv) return fail(CPM_ERR_INVALID_ARG, "server_step: null server");
    const int nb = (int)sv->solvers.size();
    cudaStream_t caller = stream();
    int n_fin = 0;
    for (int b = 0; b < nb; ++b)  // a previous cpm_server_step_async's launches
        if (sv->inflight[b]) CPM_TRY(server_harvest(sv, b, caller, &n_fin));
    for (int b = 0; b < nb; ++b) CPM_TRY(server_launch(sv, b));
    for (int b = 0; b < nb; ++b) CPM_TRY(server_harvest(sv, b, caller, &n_fin));
    for (int b = 0; b < nb; ++b) CPM_CUDA_TRY(cudaEventSynchronize(sv->res_ev[b]));
    server_counts(sv, n_fin, active, queued, finished);
    return 0;
}

// The same round, pipelined: harvest what the previous call launched, then admit
// and launch and return without waiting, so the caller's polls (the host copies
// of the finished solutions) overlap the graphs just launched.  A call that
// leaves nothing busy waits for its own results, as cpm_server_step does.
extern "C" int cpm_server_step_async(cpm_server_t sv, int32_t *active, int32_t *queued, int32_t *finished) {
    if (!sv) return fail(CPM_ERR_INVALID_ARG, "server_step_async: null server");
    const int nb = (int)sv->solvers.size();
    cudaStream_t caller = stream();
    int n_fin = 0;
    for (int b = 0; b < nb; ++b)
        if (sv->inflight[b]) CPM_TRY(server_harvest(sv, b, caller, &n_fin));
    for (int b = 0; b < nb; ++b) CPM_TRY(server_launch(sv, b));
    int n_busy = 0;
    for (auto &bz : sv->busy) n_busy += bz.used;
    if (n_busy == 0 && sv->queue.empty()) {  // idle: nothing left to overlap with
        for (int b = 0; b < nb; ++b) CPM_TRY(server_harvest(sv, b, caller, &n_fin));
        for (int b = 0; b < nb; ++b) CPM_CUDA_TRY(cudaEventSynchronize(sv->res_ev[b]));
    }
    server_counts(sv, n_fin, active, queued, finished);
    return 0;
}

extern "C" int cpm_server_poll(cpm_server_t sv, int64_t *tag, double *x, cpm_solve_stats *stats, double *latency) {
    if (!sv) return fail(CPM_ERR_INVALID_ARG, "server_poll: null server");
    if (sv->done.empty()) return 0;
    cpm_server_s::Done &d = sv->done.front();
    if (tag) *tag = d.tag;
    if (x && d.pend) {
        CPM_CUDA_TRY(cudaEventSynchronize(sv->res_ev[d.pb]));
        memcpy(x, d.pend, sizeof(double) * sv->solvers[0]->D);
    } else if (x && !d.x.empty()) {
        memcpy(x, d.x.data(), sizeof(double) * d.x.size());
    }
    if (stats) *stats = d.st;
    if (latency) *latency = d.latency;
    sv->done.pop_front();
    return 1;
}

extern "C" int cpm_server_destroy(cpm_server_t sv) {
    delete sv;
    return 0;
}

extern "C" int64_t cpm_server_device_bytes(cpm_opset_t op) {
    if (!op) return -1;
    const int64_t D = op->D;
    // per 32-slot batch, the larger of the two precisions: FP32 Krylov vectors (10) + FP64
    // b, x, r, E~x (4), or FP64 Krylov vectors (8) + the same 4; staging; reduction scratch
    return D * 32 * (12 * 8 + 8) + D * (8 + 4) + (int64_t)(1 << 20);
}

// ================================================================= apply

extern "C" int cpm_apply(cpm_opset_t op, double m, double n, int32_t k, const double *x, double *y) {
    if (!op || !x || !y || k < 1) return fail(CPM_ERR_INVALID_ARG, "invalid apply arguments");
    const int64_t D = op->D;
    DBuf<double> dx, dt, dy;
    CPM_TRY(dx.alloc(D));
    CPM_TRY(dt.alloc(D));
    CPM_TRY(dy.alloc(D));
    auto v = op->view<double>();
    for (int j = 0; j < k; ++j) {
        CPM_CUDA_TRY(cudaMemcpyAsync(dx.p, x + (size_t)j * D, D * 8, cudaMemcpyHostToDevice, stream()));
        launch_epass<double, 1>(v, nullptr, -1, dx.p, dt.p, stream());
        k_lpass<double, 1><<<row_grid(D, 1), BS, 0, stream()>>>(v, m, n, dx.p, dt.p, dy.p);
        CPM_CUDA_TRY(cudaGetLastError());
        CPM_CUDA_TRY(cudaMemcpyAsync(y + (size_t)j * D, dy.p, D * 8, cudaMemcpyDeviceToHost, stream()));
    }
    CPM_CUDA_TRY(cudaStreamSynchronize(stream()));
    return 0;
}

// identity rows of Lfull hold 1 on the diagonal (SetIdentityRows): u + dt Lfull u
// is (1 + dt) u there
__global__ void k_scale_ident(const int32_t *__restrict__ ident, int64_t n_ident, double f, const double *__restrict__ u,
                              double *__restrict__ v) {
    const int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (q < n_ident) v[ident[q]] = f * u[ident[q]];
}

// explicit heat step u <- Efull (u + dt Lfull u) (HeatWithIBC::TimeStep, method 0,
// problems/HeatWithIBC.cpp:129-132): the L pass with the row's own vector as its
// neighbour input, the identity rows scaled by 1 + dt, then the E pass (identity
// rows copy, as Efull's unit diagonal there)
extern "C" int cpm_explicit_step(cpm_opset_t op, double dt, int32_t k, const double *u, double *u_out) {
    if (!op || !u || !u_out || k < 1) return fail(CPM_ERR_INVALID_ARG, "invalid explicit step arguments");
    const int64_t D = op->D;
    DBuf<double> du, dv;
    CPM_TRY(du.alloc(D));
    CPM_TRY(dv.alloc(D));
    auto v = op->view<double>();
    for (int j = 0; j < k; ++j) {
        CPM_CUDA_TRY(cudaMemcpyAsync(du.p, u + (size_t)j * D, D * 8, cudaMemcpyHostToDevice, stream()));
        k_lpass<double, 1><<<row_grid(D, 1), BS, 0, stream()>>>(v, 1.0, dt, du.p, du.p, dv.p);
        if (v.n_ident > 0) k_scale_ident<<<nblk(v.n_ident), BS, 0, stream()>>>(v.ident, v.n_ident, 1.0 + dt, du.p, dv.p);
        CPM_CUDA_TRY(cudaGetLastError());
        launch_epass<double, 1>(v, nullptr, -1, dv.p, du.p, stream());
        CPM_CUDA_TRY(cudaGetLastError());
        CPM_CUDA_TRY(cudaMemcpyAsync(u_out + (size_t)j * D, du.p, D * 8, cudaMemcpyDeviceToHost, stream()));
    }
    CPM_CUDA_TRY(cudaStreamSynchronize(stream()));
    return 0;
}

// Gray-Scott reaction terms from the old u, v: un += dt (-u v^2 + F (1 - u)),
// vn += dt (u v^2 - (F + k) v)   (problems/ReactionDiffusionWithIBC.cpp:104-110)
__global__ void k_gray_scott(int64_t D, double dt, double F, double k, const double *__restrict__ u, const double *__restrict__ v,
                             double *__restrict__ un, double *__restrict__ vn) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= D) return;
    const double uv2 = u[i] * v[i] * v[i];
    un[i] += dt * (-uv2 + F * (1.0 - u[i]));
    vn[i] += dt * (uv2 - (F + k) * v[i]);
}

// ReactionDiffusionWithIBC::TimeStep (problems/ReactionDiffusionWithIBC.cpp:93-117)
// before its Dirichlet values: u <- Efull (u + nu_u dt Lfull u + dt R_u(u, v)),
// v <- Efull (v + nu_v dt Lfull v + dt R_v(u, v)), nu_u = (dx / 3)^2, nu_v = nu_u / 3
extern "C" int cpm_gray_scott_step(cpm_opset_t op, double dt, double F, double k, double *u, double *v) {
    if (!op || !u || !v) return fail(CPM_ERR_INVALID_ARG, "invalid reaction-diffusion step arguments");
    const int64_t D = op->D;
    const double nu_u = 1.0 / ((3.0 / op->dx) * (3.0 / op->dx)), nu_v = nu_u / 3.0;
    DBuf<double> du, dv, dun, dvn;
    CPM_TRY(du.upload(u, D));
    CPM_TRY(dv.upload(v, D));
    CPM_TRY(dun.alloc(D));
    CPM_TRY(dvn.alloc(D));
    auto w = op->view<double>();
    k_lpass<double, 1><<<row_grid(D, 1), BS, 0, stream()>>>(w, 1.0, nu_u * dt, du.p, du.p, dun.p);
    k_lpass<double, 1><<<row_grid(D, 1), BS, 0, stream()>>>(w, 1.0, nu_v * dt, dv.p, dv.p, dvn.p);
    if (w.n_ident > 0) {
        k_scale_ident<<<nblk(w.n_ident), BS, 0, stream()>>>(w.ident, w.n_ident, 1.0 + nu_u * dt, du.p, dun.p);
        k_scale_ident<<<nblk(w.n_ident), BS, 0, stream()>>>(w.ident, w.n_ident, 1.0 + nu_v * dt, dv.p, dvn.p);
    }
    k_gray_scott<<<nblk(D), BS, 0, stream()>>>(D, dt, F, k, du.p, dv.p, dun.p, dvn.p);
    CPM_CUDA_TRY(cudaGetLastError());
    launch_epass<double, 1>(w, nullptr, -1, dun.p, du.p, stream());
    launch_epass<double, 1>(w, nullptr, -1, dvn.p, dv.p, stream());
    CPM_CUDA_TRY(cudaGetLastError());
    CPM_CUDA_TRY(cudaMemcpyAsync(u, du.p, D * 8, cudaMemcpyDeviceToHost, stream()));
    CPM_CUDA_TRY(cudaMemcpyAsync(v, dv.p, D * 8, cudaMemcpyDeviceToHost, stream()));
    CPM_CUDA_TRY(cudaStreamSynchronize(stream()));
    return 0;
}

extern "C" int cpm_apply_device(cpm_opset_t op, double m, double n, int32_t kslots, int32_t fp32, const void *x_dev, void *t_dev,
                                void *y_dev) {
    if (!op || !x_dev || !t_dev || !y_dev || (kslots != 1 && kslots != 32))
        return fail(CPM_ERR_INVALID_ARG, "apply_device: null pointer or kslots not 1 / 32");
    const int64_t D = op->D;
    cudaStream_t st = stream();
    if (fp32) {
        auto v = op->view<float>();
        const float *x = (const float *)x_dev;
        float *t = (float *)t_dev, *y = (float *)y_dev;
        if (kslots == 1) {
            launch_epass<float, 1>(v, nullptr, -1, x, t, st);
            k_lpass<float, 1><<<row_grid(D, 1), BS, 0, st>>>(v, (float)m, (float)n, x, t, y);
        } else {
            launch_epass<float, 32>(v, nullptr, -1, x, t, st);
            if (lpass4_ok(D, x, t, y))
                if (v.ov_ptr)
                    k_lpass4<true><<<row_grid(D, 32), BS, 0, st>>>(v, (float)m, (float)n, x, t, y);
                else
                    k_lpass4<false><<<row_grid(D, 32), BS, 0, st>>>(v, (float)m, (float)n, x, t, y);
            else
                k_lpass<float, 32><<<row_grid(D, 32), BS, 0, st>>>(v, (float)m, (float)n, x, t, y);
        }
    } else {
        auto v = op->view<double>();
        const double *x = (const double *)x_dev;
        double *t = (double *)t_dev, *y = (double *)y_dev;
        if (kslots == 1) {
            launch_epass<double, 1>(v, nullptr, -1, x, t, st);
            k_lpass<double, 1><<<row_grid(D, 1), BS, 0, st>>>(v, m, n, x, t, y);
        } else {
            launch_epass<double, 32>(v, nullptr, -1, x, t, st);
            k_lpass<double, 32><<<row_grid(D, 32), BS, 0, st>>>(v, m, n, x, t, y);
        }
    }
    count_launches(1 + (kslots == 32 ? (fp32 ? epass_kernels<float, 32>(op->view<float>(), (const float *)x_dev)
                                              : epass_kernels<double, 32>(op->view<double>(), (const double *)x_dev))
                                      : 1));
    CPM_CUDA_TRY(cudaGetLastError());
    return 0;
}

// ================================================================= launch-shape autotuner
// Times each 32-slot E-pass kernel of one operator over candidate grid sizes
// (blocks per SM of its grid-stride loop) on scratch vectors, keeps the
// fastest with the operator, and reports the times.  The grid sizes change no
// arithmetic: every row and slot is summed by the same code in the same order.
namespace {
__global__ void k_tune_fill(int64_t n, float *__restrict__ a, double *__restrict__ b) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float v = (float)((i * 2654435761ull) % 2001ull) * 1e-3f - 1.0f;  // deterministic values in [-1, 1]
    if (a) a[i] = v;
    if (b) b[i] = (double)v;
}

template <class F>
float time_launches(cudaStream_t st, int reps, F launch) {
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    launch();  // warm
    cudaEventRecord(e0, st);
    for (int r = 0; r < reps; ++r) launch();
    cudaEventRecord(e1, st);
    cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return ms * 1000.f / (float)reps;
}
}  // namespace

extern "C" int cpm_opset_set_launch(cpm_opset_t op, int32_t e32_bps, int32_t patch_bps, int32_t e64_bps) {
    if (!op || e32_bps < 0 || patch_bps < 0 || e64_bps < 0 || e32_bps > 1024 || patch_bps > 1024 || e64_bps > 1024)
        return fail(CPM_ERR_INVALID_ARG, "opset_set_launch: null operator or blocks per SM outside 0..1024");
    op->e32_bps = e32_bps;
    op->patch_bps = patch_bps;
    op->e64_bps = e64_bps;
    return 0;
}

extern "C" int cpm_opset_autotune(cpm_opset_t op, int32_t reps, int32_t with_fp64, cpm_tune_result *out) {
    if (!op || reps < 1 || reps > 1000) return fail(CPM_ERR_INVALID_ARG, "opset_autotune: null operator or reps outside 1..1000");
    const int64_t D = op->D, n = D * 32;
    cudaStream_t st = stream();
    DBuf<float> x32, t32;
    DBuf<double> x64, t64;
    CPM_TRY(x32.alloc(n));
    CPM_TRY(t32.alloc(n));
    if (with_fp64) {
        CPM_TRY(x64.alloc(n));
        CPM_TRY(t64.alloc(n));
    }
    k_tune_fill<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(n, x32.p, with_fp64 ? x64.p : nullptr);
    CPM_CUDA_TRY(cudaGetLastError());
    cpm_tune_result res;
    memset(&res, 0, sizeof(res));
    const int sms = sm_count();
    const int e32c[] = {8, 16, 24, 32, 48, 64, 96, 128}, pc[] = {4, 8, 16, 32, 64, 128}, e64c[] = {4, 8, 16, 32, 64};
    const OpView<float> v32 = op->view<float>();
    auto pick = [&](const int *c, int nc, int dflt, auto launch_with, float &best_us, float &dflt_us, int32_t &best) {
        best_us = 0.f;
        dflt_us = 0.f;
        best = dflt;
        for (int i = 0; i < nc; ++i) {
            const float us = time_launches(st, reps, [&] { launch_with(c[i]); });
            if (c[i] == dflt) dflt_us = us;
            if (best_us == 0.f || us < best_us) {
                best_us = us;
                best = c[i];
            }
        }
        // keep the default unless another shape is at least 2 % faster
        if (dflt_us > 0.f && best_us > 0.98f * dflt_us) {
            best = dflt;
            best_us = dflt_us;
        }
    };
    if (op->n_grp > 0) {
        pick(e32c, 8, E32_BPS, [&](int bps) {
            const int64_t blocks = std::max<int64_t>(1, std::min<int64_t>((v32.n_grp + 3) / 4, (int64_t)bps * sms));
            k_epass32w<<<(unsigned)blocks, 128, 0, st>>>(v32, nullptr, -1, x32.p, t32.p);
        }, res.e32_us, res.e32_default_us, res.e32_blocks_per_sm);
    }
    if (op->n_pl > 0) {
        pick(pc, 6, PATCH_BPS, [&](int bps) {
            const int64_t blocks = std::max<int64_t>(1, std::min<int64_t>((v32.n_pl + 3) / 4, (int64_t)bps * sms));
            if (v32.ov_ptr)
                k_epatch32<float, true><<<(unsigned)blocks, 128, 0, st>>>(v32, nullptr, -1, x32.p, t32.p);
            else
                k_epatch32<float, false><<<(unsigned)blocks, 128, 0, st>>>(v32, nullptr, -1, x32.p, t32.p);
        }, res.patch_us, res.patch_default_us, res.patch_blocks_per_sm);
    }
    if (with_fp64 && op->n_grp > 0) {
        const OpView<double> v64 = op->view<double>();
        pick(e64c, 5, E64_BPS, [&](int bps) {
            const int64_t blocks = std::max<int64_t>(1, std::min<int64_t>(v64.n_grp, (int64_t)bps * sms));
            k_epass32s<double><<<(unsigned)blocks, 128, 0, st>>>(v64, nullptr, -1, x64.p, t64.p);
        }, res.e64_us, res.e64_default_us, res.e64_blocks_per_sm);
    }
    CPM_CUDA_TRY(cudaGetLastError());
    CPM_CUDA_TRY(cudaStreamSynchronize(st));
    op->e32_bps = res.e32_blocks_per_sm;
    op->patch_bps = res.patch_blocks_per_sm;
    if (with_fp64) op->e64_bps = res.e64_blocks_per_sm;
    if (out) *out = res;
    return 0;
}

// ================================================================= allocation-free apply
// The E~x scratch of cpm_apply_device_noalloc: one fixed array per device,
// shared by every call (see include/cpm_gpu.h for the contract).
static __device__ __align__(256) unsigned char g_noalloc_scratch[CPM_NOALLOC_SCRATCH_BYTES];

namespace {
std::mutex g_noalloc_mu;
constexpr int kMaxDevices = 64;
void *g_noalloc_ptr[kMaxDevices] = {nullptr};

// device address of the scratch array on the current device, looked up once per device
int noalloc_scratch(void **out) {
    int dev = 0;
    CPM_CUDA_TRY(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDevices) return fail(CPM_ERR_INVALID_ARG, "apply_device_noalloc: device index out of range");
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    if (!g_noalloc_ptr[dev]) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p)
            return fail(CPM_ERR_CUDA, std::string("apply_device_noalloc: cudaGetSymbolAddress: ") + cudaGetErrorString(e));
        g_noalloc_ptr[dev] = p;
    }
    *out = g_noalloc_ptr[dev];
    return 0;
}
}  // namespace

extern "C" int cpm_apply_device_noalloc(cpm_opset_t op, double m, double n, int32_t kslots, int32_t fp32, const void *x_dev,
                                        void *y_dev) {
    if (!op || !x_dev || !y_dev || (kslots != 1 && kslots != 32))
        return fail(CPM_ERR_INVALID_ARG, "apply_device_noalloc: null pointer or kslots not 1 / 32");
    const size_t need = (size_t)op->D * (size_t)kslots * (fp32 ? sizeof(float) : sizeof(double));
    if (need > (size_t)CPM_NOALLOC_SCRATCH_BYTES)
        return fail(CPM_ERR_INVALID_ARG, "apply_device_noalloc: scratch of " + std::to_string(need) +
                                             " bytes exceeds the fixed " + std::to_string(CPM_NOALLOC_SCRATCH_BYTES) +
                                             "-byte array; use cpm_apply_device with caller scratch");
    void *t = nullptr;
    CPM_TRY(noalloc_scratch(&t));
    const int64_t D = op->D;
    cudaStream_t st = stream();
    if (fp32) {
        auto v = op->view<float>();
        const float *x = (const float *)x_dev;
        float *tt = (float *)t, *y = (float *)y_dev;
        if (kslots == 1) {
            launch_epass<float, 1>(v, nullptr, -1, x, tt, st);
            k_lpass<float, 1><<<row_grid(D, 1), BS, 0, st>>>(v, (float)m, (float)n, x, tt, y);
        } else {
            launch_epass<float, 32>(v, nullptr, -1, x, tt, st);
            if (lpass4_ok(D, x, tt, y))
                if (v.ov_ptr)
                    k_lpass4<true><<<row_grid(D, 32), BS, 0, st>>>(v, (float)m, (float)n, x, tt, y);
                else
                    k_lpass4<false><<<row_grid(D, 32), BS, 0, st>>>(v, (float)m, (float)n, x, tt, y);
            else
                k_lpass<float, 32><<<row_grid(D, 32), BS, 0, st>>>(v, (float)m, (float)n, x, tt, y);
        }
    } else {
        auto v = op->view<double>();
        const double *x = (const double *)x_dev;
        double *tt = (double *)t, *y = (double *)y_dev;
        if (kslots == 1) {
            launch_epass<double, 1>(v, nullptr, -1, x, tt, st);
            k_lpass<double, 1><<<row_grid(D, 1), BS, 0, st>>>(v, m, n, x, tt, y);
        } else {
            launch_epass<double, 32>(v, nullptr, -1, x, tt, st);
            k_lpass<double, 32><<<row_grid(D, 32), BS, 0, st>>>(v, m, n, x, tt, y);
        }
    }
    count_launches(1 + (kslots == 32 ? (fp32 ? epass_kernels<float, 32>(op->view<float>(), (const float *)x_dev)
                                              : epass_kernels<double, 32>(op->view<double>(), (const double *)x_dev))
                                      : 1));
    CPM_CUDA_TRY(cudaGetLastError());
    return 0;
}
