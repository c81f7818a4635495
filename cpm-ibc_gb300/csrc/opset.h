// Operator set: device rows of Lfull / Efull (with the IBC patch) and the
// device-side row functions of the closest-point operator.
#pragma once

#include <memory>

#include "cpm_internal.h"

namespace cpm {

enum RowFlags : uint8_t {
    F_IDENT = 1,   // identity row: t = x, y = x
    F_EMOVE = 2,   // E row has columns moved to IBC DOF columns
    F_LMOVE = 4,   // tube row whose 7-point L row has moved neighbours
    F_LCSR = 8,    // L row stored as CSR (IBC DOF rows)
    F_ENEG = 16,   // E row negated (2nd-order Dirichlet DOF rows)
    F_EXTRA = 32,  // E row has one extra entry (2 * Dirichlet value)
    F_SLOTP = 64,  // tube row with per-slot patch records (a batch with one point IBC per slot)
    F_OVL = 128,   // tube row with entries that move to more than one IBC (extra targets)
};

// Device view of an operator set in one arithmetic type: the rows of E and L
// (bulk stencils, IBC patches), the apply schedule (rows sorted into base
// groups, identity rows, neighbour table) and the per-slot patches of a batch.
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
    const int32_t *nbr6;    // D x 6: each row's L columns (moves applied, -1 absent); all rows'
                            // L rows are Ldiag on the diagonal and Loff off it
    const int32_t *ord;     // non-identity rows sorted by base point (stable in row order)
    const int32_t *grp;     // base groups: ord[grp[g] .. grp[g+1]) share one base point
    const int32_t *gcols;   // 64 bulk stencil columns per group, s = 16 i + 4 j + k
    const T *w_ord;         // weights of ord[p] at 12 p (sorted copy: coalesced per group)
    const uint8_t *fl_ord;  // flags of ord[p]
    const int32_t *ident;   // identity rows
    // IBC patch list of the rows whose E row differs from the bulk stencil:
    // t_r = sign (bulk + sum_e w_e (x[new_e] - x[old_e])) + xval x[xcol]
    const int32_t *pl_row, *pl_off, *pl_xcol;  // n_pl rows; entries pl_off[i] .. pl_off[i+1]
    const uint8_t *pl_neg;                    // bit 0: negated (2nd-order Dirichlet DOF rows); bit 1: E extras (F_OVL)
    const T *pl_xval;
    const int32_t *pe_new, *pe_old;           // moved column and the bulk column it replaces
    const T *pe_w;                            // stencil weight (wx_i wy_j) wz_k of the moved point
    int64_t n_ord, n_grp, n_ident, n_pl;
    // per-slot patches of a batch whose slots each carry their own point IBC
    // (cpm_geodesic_batch_*): row r's records sp_rec[sp_ptr[r] .. sp_ptr[r + 1]),
    // {slot, 0 E entry / 1 L entry, the column it replaces, the slot's DOF column};
    // E entries carry the stencil weight.  Null when the operator has none.
    const int32_t *sp_ptr;
    const int4 *sp_rec;
    const T *sp_w;
    const int32_t *sp_rows;                   // rows with records
    int64_t n_sp_rows;
    // extra targets of the F_OVL rows (patch index pi): an entry that lies across
    // several IBCs moves to every one of their DOF columns (MoveToIBCColumns keeps
    // one copy per IBC), the first in the moved list, the others here.  E extras
    // ov_col[ov_ptr[2 pi] .. ov_ptr[2 pi + 1]) with stencil weight ov_w, L extras
    // ov_col[ov_ptr[2 pi + 1] .. ov_ptr[2 pi + 2]) with weight Loff.
    const int32_t *ov_ptr, *ov_col;
    const T *ov_w;
    // launch shapes of the 32-slot E passes, blocks per SM (0: the built-in
    // defaults; cpm_opset_autotune / cpm_opset_set_launch).  Never the arithmetic.
    int e32_bps, patch_bps, e64_bps;
};

// the per-slot L corrections of row r, slot s (K-wide batch): a moved neighbour
// reads the slot's DOF column of t instead of the tube node's
template <class T, int K>
__device__ __forceinline__ T slot_l_correction(const OpView<T> &op, int64_t r, int s, T n, const T *__restrict__ t) {
    T c = 0;
    for (int e = op.sp_ptr[r]; e < op.sp_ptr[r + 1]; ++e) {
        const int4 rec = op.sp_rec[e];
        if (rec.x == s && rec.y == 1) c += t[(int64_t)rec.w * K + s] - t[(int64_t)rec.z * K + s];
    }
    return n * (op.Loff * c);
}

// sum of x (K-wide, slot s) at an F_OVL row's E extras, weighted
template <class T, int K>
__device__ __forceinline__ T ovl_e_sum(const int32_t *ov_ptr, const int32_t *ov_col, const T *ov_w, int pi, int s,
                                       const T *__restrict__ x) {
    T a = 0;
    for (int e = ov_ptr[2 * pi]; e < ov_ptr[2 * pi + 1]; ++e) a += ov_w[e] * x[(int64_t)ov_col[e] * K + s];
    return a;
}

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
    if (fl & (F_EMOVE | F_EXTRA | F_OVL)) {
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
    if (fl & F_OVL) acc += ovl_e_sum<T, K>(op.ov_ptr, op.ov_col, op.ov_w, pi, s, x);
    if (fl & F_ENEG) acc = -acc;
    if (fl & F_EXTRA) acc += op.p_xval[pi] * x[(int64_t)op.p_xcol[pi] * K + s];
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
    if (fl & (F_EMOVE | F_EXTRA | F_OVL)) {
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
    if (fl & F_OVL) acc += ovl_e_sum<T, K>(op.ov_ptr, op.ov_col, op.ov_w, pi, s, x);
    if (fl & F_ENEG) acc = -acc;
    if (fl & F_EXTRA) acc += op.p_xval[pi] * x[(int64_t)op.p_xcol[pi] * K + s];
    return acc;
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

// Four-warp-per-group E pass for a 32-slot batch (stencil split by planes).
// Warp w holds the 16 nodes of plane i = w of the group's 4^3 stencil (lane =
// slot), evaluates wx_w * sum_j wy_j sum_k wz_k x for every row of the group,
// and the four planes are summed through shared memory.  16 registers per
// plane instead of 64 keep ~4x more warps resident to hide gather latency.
// Every row gets the bulk stencil; rows on the IBC patch list are corrected
// afterwards (k_epatch32).
constexpr int EG_ROWS = 32;  // rows per shared-memory chunk of a group
template <class T>
struct EGShared {
    T part[4][EG_ROWS][32];
    alignas(16) T w[EG_ROWS * 12];
    int rows[EG_ROWS];
};

// packed FP32 pairs (f32x2 arithmetic, one instruction for two rows)
__device__ __forceinline__ uint64_t f2_pack(float lo, float hi) {
    uint64_t r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(lo), "f"(hi));
    return r;
}
__device__ __forceinline__ void f2_unpack(uint64_t v, float &lo, float &hi) {
    asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(v));
}
__device__ __forceinline__ uint64_t f2_fma(uint64_t a, uint64_t b, uint64_t c) {
    uint64_t d;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
    return d;
}
__device__ __forceinline__ uint64_t f2_mul(uint64_t a, uint64_t b) {
    uint64_t d;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}

__device__ __forceinline__ uint64_t f2_add(uint64_t a, uint64_t b) {
    uint64_t d;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ uint64_t f2_sub(uint64_t a, uint64_t b) {
    uint64_t d;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}

// round-to-nearest fma and difference, never re-associated by the compiler
__device__ __forceinline__ float fma_rn(float a, float b, float c) { return __fmaf_rn(a, b, c); }
__device__ __forceinline__ double fma_rn(double a, double b, double c) { return __fma_rn(a, b, c); }
__device__ __forceinline__ float sub_rn(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ double sub_rn(double a, double b) { return __dsub_rn(a, b); }

// four consecutive values from 16-byte aligned shared memory, as vector loads
__device__ __forceinline__ void lds4(const float *p, float (&o)[4]) {
    const float4 v = *(const float4 *)p;
    o[0] = v.x;
    o[1] = v.y;
    o[2] = v.z;
    o[3] = v.w;
}
__device__ __forceinline__ void lds4(const double *p, double (&o)[4]) {
    const double2 a = *(const double2 *)p, b = *(const double2 *)(p + 2);
    o[0] = a.x;
    o[1] = a.y;
    o[2] = b.x;
    o[3] = b.y;
}

// the 16 columns of plane `warp` of group g: four 16-byte loads every lane makes alike
__device__ __forceinline__ void e_group_cols(const int32_t *gcols, int64_t g, int warp, int (&col)[16]) {
    const int4 *gc = (const int4 *)(gcols + 64 * g + 16 * warp);
#pragma unroll
    for (int v = 0; v < 4; ++v) {
        const int4 c = __ldg(gc + v);
        col[4 * v] = c.x;
        col[4 * v + 1] = c.y;
        col[4 * v + 2] = c.z;
        col[4 * v + 3] = c.w;
    }
}
// the plane's 16 x values of this lane's slot (inactive slots issue no memory requests)
template <class T>
__device__ __forceinline__ void e_group_x(const T *__restrict__ x, const int (&col)[16], int lane, bool act, T (&xb)[16]) {
#pragma unroll
    for (int q = 0; q < 16; ++q) xb[q] = act ? x[(uint32_t)col[q] * 32u + lane] : T(0);
}

// rows ord[p0 .. p1) of group g from the plane's x values xb
template <class T>
__device__ __forceinline__ void e_group_split(const OpView<T> &op, int p0, int p1, int warp, int lane, bool act, EGShared<T> &sh,
                                              const T (&xb)[16], T *__restrict__ t) {
    const int tid = warp * 32 + lane;
    for (int c0 = p0; c0 < p1; c0 += EG_ROWS) {
        const int nr = min(p1 - c0, EG_ROWS);
        if constexpr (sizeof(T) == 4) {
            // FP32: rows in pairs with packed f32x2 arithmetic.  The chunk's weights
            // are staged pair-interleaved (component c of rows 2p, 2p+1 at
            // 24 p + 2 c, 24 p + 2 c + 1), zero for the odd row of a last pair.
            const int nr2 = nr + (nr & 1);
            for (int e = tid; e < nr2 * 12; e += 128) {
                const int q = e / 12, c = e - 12 * q;
                sh.w[24 * (q >> 1) + 2 * c + (q & 1)] = q < nr ? op.w_ord[12 * (size_t)(c0 + q) + c] : T(0);
            }
            if (tid < nr) sh.rows[tid] = op.ord[c0 + tid];
            __syncthreads();
            uint64_t x2[16];
#pragma unroll
            for (int q = 0; q < 16; ++q) x2[q] = f2_pack((float)xb[q], (float)xb[q]);
            for (int q = 0; q < nr; q += 2) {
                const float *w = (const float *)sh.w + 12 * q;
                const uint64_t wx2 = *(const uint64_t *)(w + 2 * warp);
                const ulonglong2 y01 = *(const ulonglong2 *)(w + 8), y23 = *(const ulonglong2 *)(w + 12);
                const ulonglong2 z01 = *(const ulonglong2 *)(w + 16), z23 = *(const ulonglong2 *)(w + 20);
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
                float lo, hi;
                f2_unpack(f2_mul(wx2, ay2), lo, hi);
                sh.part[warp][q][lane] = (T)lo;
                if (q + 1 < nr) sh.part[warp][q + 1][lane] = (T)hi;
            }
        } else {
        // stage the chunk's sorted weights, row ids and flags (coalesced, independent loads)
        for (int e = tid; e < nr * 12; e += 128) sh.w[e] = op.w_ord[12 * (size_t)c0 + e];
        if (tid < nr) sh.rows[tid] = op.ord[c0 + tid];
        __syncthreads();
        for (int q = 0; q < nr; ++q) {
            const T *w = sh.w + 12 * q;
            const T wxi = w[warp];
            T wy[4], wz[4];
            lds4(w + 4, wy);
            lds4(w + 8, wz);
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
        }
        __syncthreads();
        for (int q = warp; q < nr; q += 4) {
            const int r = sh.rows[q];
            const T acc = ((sh.part[0][q][lane] + sh.part[1][q][lane]) + sh.part[2][q][lane]) + sh.part[3][q][lane];
            if (act) t[(uint32_t)r * 32u + lane] = acc;
        }
        __syncthreads();
    }
}

// The extra L targets of an F_OVL row r (OpView::ov_*), added to a finished
// row as n Loff sum_e t_e: after the row's own sum, when its neighbour columns
// are no longer live, so the row loops of operators without overlaps keep
// their registers.
template <class T, int K>
__device__ __forceinline__ T ovl_l_term(const OpView<T> &op, int64_t r, int s, T n, const T *__restrict__ t) {
    const int pi = op.patch[r];
    T a = 0;
    for (int e = op.ov_ptr[2 * pi + 1]; e < op.ov_ptr[2 * pi + 2]; ++e) a += t[(int64_t)op.ov_col[e] * K + s];
    return n * (op.Loff * a);
}

// y_r = m x_r + n (Ldiag x_r + Loff sum_d t_{c_d}), identity rows y = x
// (GeneralizedBiCGStabSystem::Multiply, src/GeneralizedBiCGStabSystem.h:191-233)
// for slot s of a K-wide row-major batch and U rows at once: the flags, x and
// neighbour columns of all U rows are loaded first, then their 6 U gathers of
// t, so U rows' memory requests are in flight together.  Rows >= D produce
// nothing; an inactive slot (act false) reads nothing.
template <class T, int K, int U>
__device__ __forceinline__ void l_rows(const OpView<T> &op, const int64_t (&r)[U], int s, T m, T n, const T *__restrict__ x,
                                       const T *__restrict__ t, bool act, T (&y)[U]) {
    uint8_t fl[U];
    T xr[U];
    int c[U][6];
#pragma unroll
    for (int u = 0; u < U; ++u) {
        const bool ok = r[u] < op.D;
        fl[u] = ok ? __ldg(op.flags + r[u]) : (uint8_t)F_IDENT;
        xr[u] = (ok && act) ? x[r[u] * K + s] : T(0);
        int2 a = make_int2(-1, -1), b = a, e = a;
        if (ok) {
            a = __ldg((const int2 *)(op.nbr6 + 6 * r[u]));
            b = __ldg((const int2 *)(op.nbr6 + 6 * r[u] + 2));
            e = __ldg((const int2 *)(op.nbr6 + 6 * r[u] + 4));
        }
        c[u][0] = a.x;
        c[u][1] = a.y;
        c[u][2] = b.x;
        c[u][3] = b.y;
        c[u][4] = e.x;
        c[u][5] = e.y;
    }
    if constexpr (sizeof(T) == 8) {
#pragma unroll
        for (int u = 0; u < U; ++u) {
            T off = 0;
#pragma unroll
            for (int d = 0; d < 6; ++d)
                if (c[u][d] >= 0 && act && !(fl[u] & F_IDENT)) off += t[(int64_t)c[u][d] * K + s];
            y[u] = (fl[u] & F_IDENT) ? xr[u] : m * xr[u] + n * (op.Ldiag * xr[u] + op.Loff * off);
            if ((fl[u] & F_SLOTP) && act) y[u] += slot_l_correction<T, K>(op, r[u], s, n, t);
        }
    } else {
        // FP32: the same row as Loff (sum_d (t_d - x) + (k - 6) x) with k present
        // neighbours (Ldiag = -6 Loff).  The differences of a smooth field are
        // exact, so the O(1/dx^2) terms no longer cancel in FP32 arithmetic.
#pragma unroll
        for (int u = 0; u < U; ++u) {
            T off = 0;
            int k = 0;
#pragma unroll
            for (int d = 0; d < 6; ++d)
                if (c[u][d] >= 0 && act && !(fl[u] & F_IDENT)) {
                    off += t[(int64_t)c[u][d] * K + s] - xr[u];
                    ++k;
                }
            off += (T)(k - 6) * xr[u];
            y[u] = (fl[u] & F_IDENT) ? xr[u] : m * xr[u] + n * (op.Loff * off);
            if ((fl[u] & F_SLOTP) && act) y[u] += slot_l_correction<T, K>(op, r[u], s, n, t);
        }
    }
#pragma unroll
    for (int u = 0; u < U; ++u)
        if ((fl[u] & F_OVL) && act) y[u] += ovl_l_term<T, K>(op, r[u], s, n, t);
}

// l_rows for 32 FP32 slots, four per thread: slots 4q .. 4q+3 of U rows, as
// two f32x2 pairs (slots 4q, 4q+1 in .x; 4q+2, 4q+3 in .y).  One 16-byte load
// per vector and row, the neighbour columns shared by the four slots, and the
// difference form of the FP32 row on slot pairs.  Rows >= D produce nothing.
// OVL: the operator has extra L targets (OpView::ov_*); only then is their
// code compiled in, so the hot kernels of other operators are unchanged.
template <int U, bool OVL>
__device__ __forceinline__ void l_rows4(const OpView<float> &op, const int64_t (&r)[U], int q, float m, float n,
                                        const float *__restrict__ x, const float *__restrict__ t, ulonglong2 (&y)[U]) {
    uint8_t fl[U];
    ulonglong2 xr[U];
    int c[U][6];
#pragma unroll
    for (int u = 0; u < U; ++u) {
        const bool ok = r[u] < op.D;
        fl[u] = ok ? __ldg(op.flags + r[u]) : (uint8_t)F_IDENT;
        xr[u] = ok ? *(const ulonglong2 *)(x + (uint32_t)r[u] * 32u + 4 * q) : make_ulonglong2(0ull, 0ull);
        int2 a = make_int2(-1, -1), b = a, e = a;
        if (!(fl[u] & F_IDENT)) {
            a = __ldg((const int2 *)(op.nbr6 + 6 * r[u]));
            b = __ldg((const int2 *)(op.nbr6 + 6 * r[u] + 2));
            e = __ldg((const int2 *)(op.nbr6 + 6 * r[u] + 4));
        }
        c[u][0] = a.x;
        c[u][1] = a.y;
        c[u][2] = b.x;
        c[u][3] = b.y;
        c[u][4] = e.x;
        c[u][5] = e.y;
    }
    const uint64_t m2 = f2_pack(m, m), n2 = f2_pack(n, n), l2 = f2_pack(op.Loff, op.Loff);
#pragma unroll
    for (int u = 0; u < U; ++u) {
        uint64_t o0 = 0ull, o1 = 0ull;  // +0.0f pairs
        int k = 0;
#pragma unroll
        for (int d = 0; d < 6; ++d)
            if (c[u][d] >= 0) {
                const ulonglong2 tv = *(const ulonglong2 *)(t + (uint32_t)c[u][d] * 32u + 4 * q);
                o0 = f2_add(o0, f2_sub(tv.x, xr[u].x));
                o1 = f2_add(o1, f2_sub(tv.y, xr[u].y));
                ++k;
            }
        const float km = (float)(k - 6);
        const uint64_t k2 = f2_pack(km, km);
        o0 = f2_fma(k2, xr[u].x, o0);
        o1 = f2_fma(k2, xr[u].y, o1);
        if (fl[u] & F_IDENT) {
            y[u] = xr[u];
        } else {
            y[u].x = f2_fma(n2, f2_mul(l2, o0), f2_mul(m2, xr[u].x));
            y[u].y = f2_fma(n2, f2_mul(l2, o1), f2_mul(m2, xr[u].y));
        }
    }
    if constexpr (OVL)
#pragma unroll
    for (int u = 0; u < U; ++u)
        if (fl[u] & F_OVL) {  // extra L targets, n Loff sum_e t_e (never an identity row)
            const int pi = op.patch[r[u]];
            uint64_t a0 = 0ull, a1 = 0ull;
            for (int e = op.ov_ptr[2 * pi + 1]; e < op.ov_ptr[2 * pi + 2]; ++e) {
                const ulonglong2 tv = *(const ulonglong2 *)(t + (uint32_t)op.ov_col[e] * 32u + 4 * q);
                a0 = f2_add(a0, tv.x);
                a1 = f2_add(a1, tv.y);
            }
            y[u].x = f2_fma(n2, f2_mul(l2, a0), y[u].x);
            y[u].y = f2_fma(n2, f2_mul(l2, a1), y[u].y);
        }
}

// caller-supplied closest points of an operator set built by cpm_opset_create_from_cp
struct CpOverrides;

}  // namespace cpm

struct cpm_opset_s {
    cpm_tube_s *tube = nullptr;  // not owned
    int64_t N = 0, D = 0, total_ibc = 0, num2 = 0, n_ibc = 0, n_patched = 0, n_moved = 0;
    int e32_bps = 0, patch_bps = 0, e64_bps = 0;  // E-pass launch shapes (see OpView)
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
    cpm::DBuf<int32_t> pl_row, pl_off, pl_xcol, pe_new, pe_old;
    cpm::DBuf<uint8_t> pl_neg;
    cpm::DBuf<double> pl_xval, pe_w;
    cpm::DBuf<float> pl_xval32, pe_w32;
    int64_t n_pl = 0, n_pe = 0;
    cpm::DBuf<double> w_ord;
    cpm::DBuf<float> w_ord32;
    cpm::DBuf<uint8_t> fl_ord;
    int64_t n_ord = 0, n_grp = 0, n_ident = 0;
    // host-side row layout for right-hand sides
    std::vector<uint8_t> h_identity;
    std::vector<int32_t> h_kind, h_ibc, h_side;
    std::vector<double> h_point;
    // IBC subsets (device tube indices, reference BFS order)
    std::vector<std::vector<int64_t>> tag_set, dof_set;
    std::vector<std::vector<double>> dof_cp, dof_cpdiff;
    // unoriented surface normals of the tube nodes (eigenvector 0 of the
    // symmetrised closest-point Jacobian), kept when IBC frames needed them
    cpm::DBuf<double> normals;
    // the IBC descriptions (vertex and segment arrays owned here), for evaluation-point queries
    std::vector<cpm_surface_desc> ibc_desc;
    std::vector<std::vector<double>> ibc_verts;
    std::vector<std::vector<int64_t>> ibc_prims;
    std::vector<int64_t> col_start, dcol_start;
    int64_t identity_rows_start = 0;
    std::shared_ptr<cpm::CpOverrides> cp_ovr;  // set by cpm_opset_create_from_cp
    // per-slot patches (a batch with one point IBC per slot)
    cpm::DBuf<int32_t> sp_ptr, sp_rows;
    cpm::DBuf<int4> sp_rec;
    cpm::DBuf<double> sp_w;
    cpm::DBuf<float> sp_w32;
    int64_t n_sp_rows = 0;
    // extra targets of entries that move to several IBCs (OpView::ov_*); the
    // host copy keeps each E extra's stencil index (s = 16 i + 4 j + k) or L
    // neighbour (d) in h_ov_s
    cpm::DBuf<int32_t> ov_ptr, ov_col;
    cpm::DBuf<double> ov_w;
    cpm::DBuf<float> ov_w32;
    std::vector<int32_t> h_ov_ptr, h_ov_col, h_ov_s;
    int64_t n_ov = 0;  // extra targets in all

    template <class T>
    cpm::OpView<T> view() const;
};

namespace cpm {
// whole-tube Jcp surface normals (eigenvector 0) of the operator's tube, uploaded to o->normals
int opset_tube_normals(cpm_opset_s *o);

// A batch of point IBCs, one per slot (the heat-method geodesic from n_src
// sources at once): the plain tube operator with M = the largest DOF count
// identity rows appended (slot k's DOF i is row N + i, holding its Dirichlet
// value) and, as per-slot patch records, each slot's moved E and L columns of
// the tube rows near its source (AddIBCExtension / AddIBCFiniteDifference of
// an order-1 Dirichlet point IBC).  info: each source's DOF subset (tube
// rows) and cp_diff, for the heat step's right-hand side.
struct PointBatchInfo {
    std::vector<std::vector<int64_t>> dof_set;
    std::vector<std::vector<double>> dof_cpdiff;
};
int opset_create_point_batch(cpm_tube_s *t, int n_src, const double *sources, cpm_opset_s **out, PointBatchInfo &info);

// E~ x of a [D][32] FP64 batch, every slot, on the library stream; slot_patches
// false leaves out a batch operator's per-slot point-IBC patches (the plain E)
int epass64_batch(const cpm_opset_s *o, bool slot_patches, const double *x, double *t);
}  // namespace cpm
