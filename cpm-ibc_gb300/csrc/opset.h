// Operator set: device rows of Lfull / Efull (with the IBC patch) and the
// device-side row functions of the closest-point operator.
#pragma once

#include "cpm_internal.h"

namespace cpm {

enum RowFlags : uint8_t {
    F_IDENT = 1,   // identity row: t = x, y = x
    F_EMOVE = 2,   // E row has columns moved to IBC DOF columns
    F_LMOVE = 4,   // tube row whose 7-point L row has moved neighbours
    F_LCSR = 8,    // L row stored as CSR (IBC DOF rows)
    F_ENEG = 16,   // E row negated (2nd-order Dirichlet DOF rows)
    F_EXTRA = 32,  // E row has one extra entry (2 * Dirichlet value)
};

template <class T>
struct OpView {
    BrickView bv;
    int64_t N, D;
    const uint32_t *key;    // tube rows: packed node triplet
    const uint32_t *base;   // D: packed base triplet of the row's interpolation stencil
    const T *w;             // 12*D tricubic 1-D weights [d][j]
    const uint8_t *flags;   // D
    const int32_t *patch;   // D: patch index or -1
    const uint64_t *p_emask;
    const int32_t *p_eoff;
    const uint8_t *p_lmask;
    const int32_t *p_loff;
    const int32_t *moved;   // moved column targets
    const int32_t *p_xcol;  // extra E entry column
    const T *p_xval;        // extra E entry value
    const int32_t *lptr;    // rows >= N: CSR of off-diagonal L entries, indexed r - N
    const int32_t *lcol;
    const T *lval;
    const T *ldiag;         // rows >= N: L diagonal
    T Ldiag, Loff;          // tube rows: -6/dx^2 and 1/dx^2
    // apply schedule
    const int32_t *nbr6;    // tube rows: the six L columns (moves applied, -1 absent)
    const int32_t *ord;     // non-identity rows sorted by base point (stable in row order)
    const int32_t *grp;     // base groups: ord[grp[g] .. grp[g+1]) share one base point
    const int32_t *gcols;   // 64 bulk stencil columns per group, s = 16 i + 4 j + k
    const T *w_ord;         // weights of ord[p] at 12 p (sorted copy: coalesced per group)
    const uint8_t *fl_ord;  // flags of ord[p]
    const int32_t *ident;   // identity rows
    int64_t n_ord, n_grp, n_ident;
};

// ---------------------------------------------------------------------------
// A 4^3 stencil based at (bi,bj,bk) touches at most 2x2x2 bricks: corner c =
// ox | oy<<1 | oz<<2 with o? = 1 when the stencil crosses into the next brick.
// Each corner's (first node, occupancy mask) is resolved once per row.
struct Corner {
    int start;
    uint64_t mask;
};

__device__ __forceinline__ Corner load_corner(const BrickView &b, int X, int Y, int Z) {
    Corner c{0, 0ull};
    if (X < b.NB && Y < b.NB && Z < b.NB) {
        int r = __ldg(&b.bmap[((size_t)X * b.NB + Y) * b.NB + Z]);
        if (r >= 0) {
            c.mask = __ldg(&b.bmask[r]);
            c.start = __ldg(&b.bstart[r]);
        }
    }
    return c;
}

__device__ __forceinline__ int corner_node(const Corner &c, int l) {
    return ((c.mask >> l) & 1ull) ? c.start + __popcll(c.mask & ((1ull << l) - 1ull)) : -1;
}

__device__ __forceinline__ Corner csel(bool p, const Corner &a, const Corner &b) { return p ? b : a; }

// a[i] for a runtime i in 0..3 without a dynamically indexed (local-memory) array
template <class T>
__device__ __forceinline__ T pick4(const T (&a)[4], int i) {
    const T lo = (i & 1) ? a[1] : a[0];
    const T hi = (i & 1) ? a[3] : a[2];
    return (i & 2) ? hi : lo;
}

// Thread-per-row gather: corners held in registers and picked with selects
// (no dynamically indexed register arrays, so nothing spills to local memory).
template <class T, int K>
__device__ __forceinline__ T e_row_thread(const OpView<T> &op, int64_t r, int s, const T *__restrict__ x) {
    const uint8_t fl = op.flags[r];
    if (fl & F_IDENT) return x[r * K + s];
    const uint32_t b = op.base[r];
    const int bi = unpack_i(b), bj = unpack_j(b), bk = unpack_k(b);
    const int X0 = bi >> 2, Y0 = bj >> 2, Z0 = bk >> 2;
    const bool cx = (bi & 3) != 0, cy = (bj & 3) != 0, cz = (bk & 3) != 0;
    Corner c0 = load_corner(op.bv, X0, Y0, Z0);
    Corner c1 = cx ? load_corner(op.bv, X0 + 1, Y0, Z0) : Corner{0, 0ull};
    Corner c2 = cy ? load_corner(op.bv, X0, Y0 + 1, Z0) : Corner{0, 0ull};
    Corner c3 = (cx && cy) ? load_corner(op.bv, X0 + 1, Y0 + 1, Z0) : Corner{0, 0ull};
    Corner c4 = cz ? load_corner(op.bv, X0, Y0, Z0 + 1) : Corner{0, 0ull};
    Corner c5 = (cx && cz) ? load_corner(op.bv, X0 + 1, Y0, Z0 + 1) : Corner{0, 0ull};
    Corner c6 = (cy && cz) ? load_corner(op.bv, X0, Y0 + 1, Z0 + 1) : Corner{0, 0ull};
    Corner c7 = (cx && cy && cz) ? load_corner(op.bv, X0 + 1, Y0 + 1, Z0 + 1) : Corner{0, 0ull};
    const T *w = op.w + 12 * r;
    T wx[4], wy[4], wz[4];
#pragma unroll
    for (int a = 0; a < 4; ++a) {
        wx[a] = w[a];
        wy[a] = w[4 + a];
        wz[a] = w[8 + a];
    }
    uint64_t emask = 0;
    int eoff = 0, pi = -1;
    if (fl & (F_EMOVE | F_EXTRA)) {
        pi = op.patch[r];
        emask = op.p_emask[pi];
        eoff = op.p_eoff[pi];
    }
    T acc = 0;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const int gi = bi + i;
        const bool ox = (gi >> 2) != X0;
        const Corner a0 = csel(ox, c0, c1), a1 = csel(ox, c2, c3), a2 = csel(ox, c4, c5), a3 = csel(ox, c6, c7);
        T ay = 0;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int gj = bj + j;
            const bool oy = (gj >> 2) != Y0;
            const Corner b0 = csel(oy, a0, a1), b1 = csel(oy, a2, a3);
            T az = 0;
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                const int gk = bk + k;
                const int sidx = 16 * i + 4 * j + k;
                const Corner cc = csel((gk >> 2) != Z0, b0, b1);
                int col;
                if ((emask >> sidx) & 1ull)
                    col = op.moved[eoff + __popcll(emask & ((1ull << sidx) - 1ull))];
                else
                    col = corner_node(cc, ((gi & 3) << 4) | ((gj & 3) << 2) | (gk & 3));
                T xv = (col >= 0) ? x[(int64_t)col * K + s] : T(0);
                az += wz[k] * xv;
            }
            ay += wy[j] * az;
        }
        acc += wx[i] * ay;
    }
    if (fl & F_ENEG) acc = -acc;
    if (fl & F_EXTRA) acc += op.p_xval[pi] * x[(int64_t)op.p_xcol[pi] * K + s];
    return acc;
}

// Warp-per-row gather for a 32-slot batch: lanes 0..7 resolve one corner brick
// each, every lane resolves the columns of stencil points lane and lane+32 and
// the warp broadcasts them with shuffles; each gather then reads one 128-byte
// row of the batch (all 32 right-hand sides of one node) — fully coalesced.
template <class T>
__device__ __forceinline__ T e_row_warp(const OpView<T> &op, int64_t r, int lane, const T *__restrict__ x) {
    const unsigned FULL = 0xffffffffu;
    const uint8_t fl = op.flags[r];
    if (fl & F_IDENT) return x[r * 32 + lane];
    const uint32_t b = op.base[r];
    const int bi = unpack_i(b), bj = unpack_j(b), bk = unpack_k(b);
    const int X0 = bi >> 2, Y0 = bj >> 2, Z0 = bk >> 2;
    Corner mine{0, 0ull};
    if (lane < 8) mine = load_corner(op.bv, X0 + (lane & 1), Y0 + ((lane >> 1) & 1), Z0 + (lane >> 2));
    uint64_t emask = 0;
    int eoff = 0, pi = -1;
    if (fl & (F_EMOVE | F_EXTRA)) {
        pi = op.patch[r];
        emask = op.p_emask[pi];
        eoff = op.p_eoff[pi];
    }
    int col2[2];
#pragma unroll
    for (int h = 0; h < 2; ++h) {
        const int sidx = lane + 32 * h;
        const int gi = bi + (sidx >> 4), gj = bj + ((sidx >> 2) & 3), gk = bk + (sidx & 3);
        const int cc = ((gi >> 2) - X0) | (((gj >> 2) - Y0) << 1) | (((gk >> 2) - Z0) << 2);
        Corner c;
        c.start = __shfl_sync(FULL, mine.start, cc);
        c.mask = ((uint64_t)__shfl_sync(FULL, (unsigned)(mine.mask >> 32), cc) << 32) |
                 (uint64_t)__shfl_sync(FULL, (unsigned)mine.mask, cc);
        int col = corner_node(c, ((gi & 3) << 4) | ((gj & 3) << 2) | (gk & 3));
        if ((emask >> sidx) & 1ull) col = op.moved[eoff + __popcll(emask & ((1ull << sidx) - 1ull))];
        col2[h] = col;
    }
    const T *w = op.w + 12 * r;
    T wx[4], wy[4], wz[4];
#pragma unroll
    for (int a = 0; a < 4; ++a) {
        wx[a] = w[a];
        wy[a] = w[4 + a];
        wz[a] = w[8 + a];
    }
    T acc = 0;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        T ay = 0;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            T az = 0;
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                const int sidx = 16 * i + 4 * j + k;
                const int col = __shfl_sync(FULL, col2[sidx >> 5], sidx & 31);
                T xv = (col >= 0) ? x[(int64_t)col * 32 + lane] : T(0);
                az += wz[k] * xv;
            }
            ay += wy[j] * az;
        }
        acc += wx[i] * ay;
    }
    if (fl & F_ENEG) acc = -acc;
    if (fl & F_EXTRA) acc += op.p_xval[pi] * x[(int64_t)op.p_xcol[pi] * 32 + lane];
    return acc;
}

// (E~ x)_r for slot s of a K-wide row-major batch (reference per-point walk;
// kept for odd widths such as the 9-wide Jacobian extension).
template <class T, int K>
__device__ __forceinline__ T e_row(const OpView<T> &op, int64_t r, int s, const T *__restrict__ x) {
    const uint8_t fl = op.flags[r];
    if (fl & F_IDENT) return x[r * K + s];
    const uint32_t b = op.base[r];
    const int bi = unpack_i(b), bj = unpack_j(b), bk = unpack_k(b);
    const T *w = op.w + 12 * r;
    T wx[4], wy[4], wz[4];
#pragma unroll
    for (int a = 0; a < 4; ++a) {
        wx[a] = w[a];
        wy[a] = w[4 + a];
        wz[a] = w[8 + a];
    }
    uint64_t emask = 0;
    int eoff = 0, pi = -1;
    if (fl & (F_EMOVE | F_EXTRA)) {
        pi = op.patch[r];
        emask = op.p_emask[pi];
        eoff = op.p_eoff[pi];
    }
    T acc = 0;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        T ay = 0;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            T az = 0;
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                const int sidx = 16 * i + 4 * j + k;
                int col;
                if ((emask >> sidx) & 1ull)
                    col = op.moved[eoff + __popcll(emask & ((1ull << sidx) - 1ull))];
                else
                    col = node_at(op.bv, bi + i, bj + j, bk + k);
                T xv = (col >= 0) ? x[(int64_t)col * K + s] : T(0);
                az += wz[k] * xv;
            }
            ay += wy[j] * az;
        }
        acc += wx[i] * ay;
    }
    if (fl & F_ENEG) acc = -acc;
    if (fl & F_EXTRA) acc += op.p_xval[pi] * x[(int64_t)op.p_xcol[pi] * K + s];
    return acc;
}

// y_r = m x_r + n (L_rr x_r + sum_{c != r} L_rc t_c), identity rows y = x
// (GeneralizedBiCGStabSystem::Multiply, src/GeneralizedBiCGStabSystem.h:191-233).
template <class T, int K>
__device__ __forceinline__ T l_row(const OpView<T> &op, int64_t r, int s, T m, T n, const T *__restrict__ x,
                                   const T *__restrict__ t) {
    const uint8_t fl = op.flags[r];
    const T xr = x[r * K + s];
    if (fl & F_IDENT) return xr;
    if (r < op.N) {
        const uint32_t kk = op.key[r];
        const int i = unpack_i(kk), j = unpack_j(kk), k = unpack_k(kk);
        uint8_t lmask = 0;
        int loff = 0;
        if (fl & F_LMOVE) {
            int pi = op.patch[r];
            lmask = op.p_lmask[pi];
            loff = op.p_loff[pi];
        }
        T off = 0;
#pragma unroll
        for (int d = 0; d < 6; ++d) {
            int col;
            if ((lmask >> d) & 1)
                col = op.moved[loff + __popc((unsigned)lmask & ((1u << d) - 1u))];
            else {
                const int di = (d == 0) - (d == 1), dj = (d == 2) - (d == 3), dk = (d == 4) - (d == 5);
                col = node_at(op.bv, i + di, j + dj, k + dk);
            }
            if (col >= 0) off += t[(int64_t)col * K + s];
        }
        return m * xr + n * (op.Ldiag * xr + op.Loff * off);
    }
    const int64_t q = r - op.N;
    T off = 0;
    for (int e = op.lptr[q]; e < op.lptr[q + 1]; ++e) off += op.lval[e] * t[(int64_t)op.lcol[e] * K + s];
    return m * xr + n * (op.ldiag[q] * xr + off);
}

// L row from the precomputed neighbour table (thread per row and slot).
template <class T, int K>
__device__ __forceinline__ T l_row_nbr(const OpView<T> &op, int64_t r, int s, T m, T n, const T *__restrict__ x,
                                       const T *__restrict__ t) {
    const uint8_t fl = op.flags[r];
    const T xr = x[r * K + s];
    if (fl & F_IDENT) return xr;
    if (r < op.N) {
        const int2 a = __ldg((const int2 *)(op.nbr6 + 6 * r));
        const int2 b = __ldg((const int2 *)(op.nbr6 + 6 * r + 2));
        const int2 c = __ldg((const int2 *)(op.nbr6 + 6 * r + 4));
        const int cols[6] = {a.x, a.y, b.x, b.y, c.x, c.y};
        T off = 0;
#pragma unroll
        for (int d = 0; d < 6; ++d)
            if (cols[d] >= 0) off += t[(int64_t)cols[d] * K + s];
        return m * xr + n * (op.Ldiag * xr + op.Loff * off);
    }
    const int64_t q = r - op.N;
    T off = 0;
    for (int e = op.lptr[q]; e < op.lptr[q + 1]; ++e) off += op.lval[e] * t[(int64_t)op.lcol[e] * K + s];
    return m * xr + n * (op.ldiag[q] * xr + off);
}

// the 12 tricubic weights of a row (48 or 96 bytes, 16-byte aligned) as vectors
__device__ __forceinline__ void load_w12(const float *w, float (&o)[12]) {
    const float4 *v = (const float4 *)w;
#pragma unroll
    for (int q = 0; q < 3; ++q) {
        float4 a = __ldg(v + q);
        o[4 * q] = a.x;
        o[4 * q + 1] = a.y;
        o[4 * q + 2] = a.z;
        o[4 * q + 3] = a.w;
    }
}
__device__ __forceinline__ void load_w12(const double *w, double (&o)[12]) {
    const double2 *v = (const double2 *)w;
#pragma unroll
    for (int q = 0; q < 6; ++q) {
        double2 a = __ldg(v + q);
        o[2 * q] = a.x;
        o[2 * q + 1] = a.y;
    }
}

// IBC patch of one row in the 32-slot group kernel: moved stencil points add
// w_s (x[moved] - x[orig]); 2nd-order Dirichlet rows are negated and add 2 g.
template <class T>
__device__ __forceinline__ T e_patch_warp(const OpView<T> &op, int r, uint8_t fl, const T (&w)[12], const int (&col2)[2],
                                          int lane, const T *__restrict__ x, T acc) {
    const unsigned FULL = 0xffffffffu;
    if (fl & (F_EMOVE | F_EXTRA)) {
        const int pi = op.patch[r];
        uint64_t em = op.p_emask[pi];
        int mo = op.p_eoff[pi];
        const T wx[4] = {w[0], w[1], w[2], w[3]}, wy[4] = {w[4], w[5], w[6], w[7]}, wz[4] = {w[8], w[9], w[10], w[11]};
        while (em) {  // warp-uniform: one row per warp
            const int s = __ffsll((long long)em) - 1;
            em &= em - 1;
            const int orig = __shfl_sync(FULL, (s < 32) ? col2[0] : col2[1], s & 31);
            const int nc = op.moved[mo++];
            const T ws = pick4(wx, s >> 4) * pick4(wy, (s >> 2) & 3) * pick4(wz, s & 3);
            acc += ws * (x[(uint32_t)nc * 32u + lane] - x[(uint32_t)orig * 32u + lane]);
        }
        if (fl & F_ENEG) acc = -acc;
        if (fl & F_EXTRA) acc += op.p_xval[pi] * x[(uint32_t)op.p_xcol[pi] * 32u + lane];
    } else if (fl & F_ENEG) {
        acc = -acc;
    }
    return acc;
}

// Warp-per-group E pass for a 32-slot batch.  Rows sharing a base point read
// the same 64 nodes: the warp gathers that 64 x 32 block once into registers
// (lane = slot; lanes 0..7 resolve the corner bricks, every lane two stencil
// columns, broadcast by shuffles) and evaluates every row of the group from
// registers with its own weights.  A row whose stencil has columns moved to
// IBC DOF columns adds w_s (x[moved] - x[orig]) per moved point.
template <class T>
__device__ __forceinline__ void e_group_warp(const OpView<T> &op, int64_t g, int lane, bool act, const T *__restrict__ x,
                                             T *__restrict__ t) {
    const unsigned FULL = 0xffffffffu;
    const int p0 = op.grp[g], p1 = op.grp[g + 1];
    const uint32_t b = op.base[op.ord[p0]];
    const int bi = unpack_i(b), bj = unpack_j(b), bk = unpack_k(b);
    const int X0 = bi >> 2, Y0 = bj >> 2, Z0 = bk >> 2;
    Corner mine{0, 0ull};
    if (lane < 8) mine = load_corner(op.bv, X0 + (lane & 1), Y0 + ((lane >> 1) & 1), Z0 + (lane >> 2));
    int col2[2];
#pragma unroll
    for (int h = 0; h < 2; ++h) {
        const int sidx = lane + 32 * h;
        const int gi = bi + (sidx >> 4), gj = bj + ((sidx >> 2) & 3), gk = bk + (sidx & 3);
        const int cc = ((gi >> 2) - X0) | (((gj >> 2) - Y0) << 1) | (((gk >> 2) - Z0) << 2);
        Corner c;
        c.start = __shfl_sync(FULL, mine.start, cc);
        c.mask = ((uint64_t)__shfl_sync(FULL, (unsigned)(mine.mask >> 32), cc) << 32) |
                 (uint64_t)__shfl_sync(FULL, (unsigned)mine.mask, cc);
        const int l = ((gi & 3) << 4) | ((gj & 3) << 2) | (gk & 3);
        // a missing node reads row 0 (tubes with missing stencil nodes are rejected at build time)
        col2[h] = ((c.mask >> l) & 1ull) ? c.start + __popcll(c.mask & ((1ull << l) - 1ull)) : 0;
    }
    // row-major [D][32] batches are addressed with 32-bit element offsets (D < 2^26)
    T xb[64];
#pragma unroll
    for (int s = 0; s < 64; ++s) xb[s] = x[(uint32_t)__shfl_sync(FULL, col2[s >> 5], s & 31) * 32u + lane];
    // two rows of the group in flight per iteration (independent load and FMA chains)
    for (int p = p0; p < p1; p += 2) {
        const bool two = p + 1 < p1;
        const int ra = op.ord[p];
        const int rb = two ? op.ord[p + 1] : ra;
        T wa[12], wb[12];
        load_w12(op.w + 12 * (size_t)ra, wa);
        load_w12(op.w + 12 * (size_t)rb, wb);
        const uint8_t fla = op.flags[ra], flb = op.flags[rb];
        T acc_a = 0, acc_b = 0;
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            T ay_a = 0, ay_b = 0;
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                T az_a = 0, az_b = 0;
#pragma unroll
                for (int k = 0; k < 4; ++k) {
                    az_a += wa[8 + k] * xb[16 * i + 4 * j + k];
                    az_b += wb[8 + k] * xb[16 * i + 4 * j + k];
                }
                ay_a += wa[4 + j] * az_a;
                ay_b += wb[4 + j] * az_b;
            }
            acc_a += wa[i] * ay_a;
            acc_b += wb[i] * ay_b;
        }
        acc_a = e_patch_warp(op, ra, fla, wa, col2, lane, x, acc_a);
        if (act) t[(uint32_t)ra * 32u + lane] = acc_a;
        if (two) {
            acc_b = e_patch_warp(op, rb, flb, wb, col2, lane, x, acc_b);
            if (act) t[(uint32_t)rb * 32u + lane] = acc_b;
        }
    }
}

// Four-warp-per-group E pass for a 32-slot batch (stencil split by planes).
// Warp w holds the 16 nodes of plane i = w of the group's 4^3 stencil (lane =
// slot), evaluates wx_w * sum_j wy_j sum_k wz_k x for every row of the group,
// and the four planes are summed through shared memory.  16 registers per
// plane instead of 64 keep ~4x more warps resident to hide gather latency.
constexpr int EG_ROWS = 32;  // rows per shared-memory chunk of a group
template <class T>
struct EGShared {
    T part[4][EG_ROWS][32];
    T w[EG_ROWS * 12];
    int cols[64];
    int rows[EG_ROWS];
    uint8_t fl[EG_ROWS];
};

template <class T>
__device__ __forceinline__ void e_group_split(const OpView<T> &op, int64_t g, int warp, int lane, bool act, EGShared<T> &sh,
                                              const T *__restrict__ x, T *__restrict__ t) {
    const unsigned FULL = 0xffffffffu;
    const int tid = warp * 32 + lane;
    const int p0 = op.grp[g], p1 = op.grp[g + 1];
    // the 16 columns of this warp's plane (lanes 16..31 duplicate lanes 0..15)
    const int sidx = 16 * warp + (lane & 15);
    const int mycol = __ldg(op.gcols + 64 * g + sidx);
    if (lane < 16) sh.cols[sidx] = mycol;
    T xb[16];
#pragma unroll
    for (int q = 0; q < 16; ++q) {
        const uint32_t cq = (uint32_t)__shfl_sync(FULL, mycol, q);
        xb[q] = act ? x[cq * 32u + lane] : T(0);  // inactive slots issue no memory requests
    }
    for (int c0 = p0; c0 < p1; c0 += EG_ROWS) {
        const int nr = min(p1 - c0, EG_ROWS);
        // stage the chunk's sorted weights, row ids and flags (coalesced, independent loads)
        for (int e = tid; e < nr * 12; e += 128) sh.w[e] = op.w_ord[12 * (size_t)c0 + e];
        if (tid < nr) {
            sh.rows[tid] = op.ord[c0 + tid];
            sh.fl[tid] = op.fl_ord[c0 + tid];
        }
        __syncthreads();
        for (int q = 0; q < nr; ++q) {
            const T *w = sh.w + 12 * q;
            const T wxi = w[warp];
            T wy[4], wz[4];
#pragma unroll
            for (int a = 0; a < 4; ++a) {
                wy[a] = w[4 + a];
                wz[a] = w[8 + a];
            }
            T ay = 0;
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                T az = 0;
#pragma unroll
                for (int k = 0; k < 4; ++k) az += wz[k] * xb[4 * j + k];
                ay += wy[j] * az;
            }
            sh.part[warp][q][lane] = wxi * ay;
        }
        __syncthreads();
        for (int q = warp; q < nr; q += 4) {
            const int r = sh.rows[q];
            T acc = ((sh.part[0][q][lane] + sh.part[1][q][lane]) + sh.part[2][q][lane]) + sh.part[3][q][lane];
            const uint8_t fl = sh.fl[q];
            if (fl & (F_EMOVE | F_EXTRA | F_ENEG)) {
                if (fl & (F_EMOVE | F_EXTRA)) {
                    const int pi = op.patch[r];
                    uint64_t em = op.p_emask[pi];
                    int mo = op.p_eoff[pi];
                    if (em) {
                        T w[12];
#pragma unroll
                        for (int a = 0; a < 12; ++a) w[a] = sh.w[12 * q + a];
                        const T wx[4] = {w[0], w[1], w[2], w[3]}, wy[4] = {w[4], w[5], w[6], w[7]},
                                wz[4] = {w[8], w[9], w[10], w[11]};
                        while (em) {  // warp-uniform: one row per warp
                            const int s = __ffsll((long long)em) - 1;
                            em &= em - 1;
                            const int nc = op.moved[mo++];
                            const T ws = pick4(wx, s >> 4) * pick4(wy, (s >> 2) & 3) * pick4(wz, s & 3);
                            acc += ws * (x[(uint32_t)nc * 32u + lane] - x[(uint32_t)sh.cols[s] * 32u + lane]);
                        }
                    }
                    if (fl & F_ENEG) acc = -acc;
                    if (fl & F_EXTRA) acc += op.p_xval[pi] * x[(uint32_t)op.p_xcol[pi] * 32u + lane];
                } else {
                    acc = -acc;
                }
            }
            if (act) t[(uint32_t)r * 32u + lane] = acc;
        }
        __syncthreads();
    }
}

// Warp-per-row L row for a 32-slot batch: lanes 0..5 read the six neighbour
// columns (or the CSR entries of an IBC DOF row, 32 at a time) and the warp
// broadcasts them.
template <class T>
__device__ __forceinline__ T l_row_warp(const OpView<T> &op, int64_t r, int lane, T m, T n, const T *__restrict__ x,
                                        const T *__restrict__ t, bool act = true) {
    const unsigned FULL = 0xffffffffu;
    // flags, x and the neighbour columns are independent loads: issue them together;
    // inactive slots issue no memory requests for x and t
    const uint8_t fl = op.flags[r];
    const T xr = act ? x[(uint32_t)r * 32u + lane] : T(0);
    int col = -1;
    if (r < op.N && lane < 6) col = __ldg(op.nbr6 + 6 * r + lane);
    if (fl & F_IDENT) return xr;
    if (r < op.N) {
        T off = 0;
#pragma unroll
        for (int d = 0; d < 6; ++d) {
            const int c = __shfl_sync(FULL, col, d);
            if (c >= 0 && act) off += t[(uint32_t)c * 32u + lane];
        }
        return m * xr + n * (op.Ldiag * xr + op.Loff * off);
    }
    const int64_t q = r - op.N;
    const int e0 = op.lptr[q], e1 = op.lptr[q + 1];
    T off = 0;
    for (int base = e0; base < e1; base += 32) {
        int c = -1;
        T v = 0;
        if (base + lane < e1) {
            c = op.lcol[base + lane];
            v = op.lval[base + lane];
        }
        const int cnt = min(32, e1 - base);
        for (int e = 0; e < cnt; ++e) {
            const int ce = __shfl_sync(FULL, c, e);
            const T ve = __shfl_sync(FULL, v, e);
            if (act) off += ve * t[(uint32_t)ce * 32u + lane];
        }
    }
    return m * xr + n * (op.ldiag[q] * xr + off);
}

}  // namespace cpm

struct cpm_opset_s {
    cpm_tube_s *tube = nullptr;  // not owned
    int64_t N = 0, D = 0, total_ibc = 0, num2 = 0, n_ibc = 0, n_patched = 0, n_moved = 0;
    double dx = 0;
    cpm::DBuf<uint32_t> base;
    cpm::DBuf<double> w;
    cpm::DBuf<float> w32;
    cpm::DBuf<uint8_t> flags;
    cpm::DBuf<int32_t> patch, p_eoff, p_loff, moved, p_xcol, lptr, lcol;
    cpm::DBuf<uint64_t> p_emask;
    cpm::DBuf<uint8_t> p_lmask;
    cpm::DBuf<double> p_xval, lval, ldiag;
    cpm::DBuf<float> p_xval32, lval32, ldiag32;
    cpm::DBuf<int32_t> nbr6, ord, grp, ident, gcols;
    cpm::DBuf<double> w_ord;
    cpm::DBuf<float> w_ord32;
    cpm::DBuf<uint8_t> fl_ord;
    int64_t n_ord = 0, n_grp = 0, n_ident = 0;
    // host-side row layout for right-hand sides
    std::vector<uint8_t> h_identity;
    std::vector<int32_t> h_kind, h_ibc;
    std::vector<double> h_point;
    // IBC subsets (device tube indices, reference BFS order)
    std::vector<std::vector<int64_t>> tag_set, dof_set;
    std::vector<std::vector<double>> dof_cp, dof_cpdiff;
    // unoriented surface normals of the tube nodes (eigenvector 0 of the
    // symmetrised closest-point Jacobian), kept when IBC frames needed them
    cpm::DBuf<double> normals;
    std::vector<int64_t> col_start, dcol_start;
    int64_t identity_rows_start = 0;

    template <class T>
    cpm::OpView<T> view() const;
};
