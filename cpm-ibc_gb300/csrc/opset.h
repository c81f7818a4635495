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

// (E~ x)_r for slot s of a K-wide row-major batch.  Separable tricubic sum
// sum_i wx_i sum_j wy_j sum_k wz_k x[node(b + (i,j,k))].
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
