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

// Warp-per-row L row for a 32-slot batch: lanes 0..5 resolve the six
// neighbours (or the CSR entries of an IBC DOF row, 32 at a time) and the
// warp broadcasts them.
template <class T>
__device__ __forceinline__ T l_row_warp(const OpView<T> &op, int64_t r, int lane, T m, T n, const T *__restrict__ x,
                                        const T *__restrict__ t) {
    const unsigned FULL = 0xffffffffu;
    const uint8_t fl = op.flags[r];
    const T xr = x[r * 32 + lane];
    if (fl & F_IDENT) return xr;
    if (r < op.N) {
        int col = -1;
        if (lane < 6) {
            const uint32_t kk = op.key[r];
            const int d = lane;
            uint8_t lmask = 0;
            int loff = 0;
            if (fl & F_LMOVE) {
                int pi = op.patch[r];
                lmask = op.p_lmask[pi];
                loff = op.p_loff[pi];
            }
            if ((lmask >> d) & 1)
                col = op.moved[loff + __popc((unsigned)lmask & ((1u << d) - 1u))];
            else
                col = node_at(op.bv, unpack_i(kk) + (d == 0) - (d == 1), unpack_j(kk) + (d == 2) - (d == 3),
                              unpack_k(kk) + (d == 4) - (d == 5));
        }
        T off = 0;
#pragma unroll
        for (int d = 0; d < 6; ++d) {
            const int c = __shfl_sync(FULL, col, d);
            if (c >= 0) off += t[(int64_t)c * 32 + lane];
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
            off += ve * t[(int64_t)ce * 32 + lane];
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
    // host-side row layout for right-hand sides
    std::vector<uint8_t> h_identity;
    std::vector<int32_t> h_kind, h_ibc;
    std::vector<double> h_point;
    // IBC subsets (device tube indices, reference BFS order)
    std::vector<std::vector<int64_t>> tag_set, dof_set;
    std::vector<std::vector<double>> dof_cp;
    std::vector<int64_t> col_start, dcol_start;
    int64_t identity_rows_start = 0;

    template <class T>
    cpm::OpView<T> view() const;
};
