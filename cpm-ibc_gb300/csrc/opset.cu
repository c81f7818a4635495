// Operator-set assembly: Lfull / Efull rows for the device operator.
//
//   no IBC:  Helpers::SetupMatrices (src/Helpers.cpp:86-93) — every tube row is
//            the regular brick stencil, nothing is stored per row but the base
//            point and the 12 weights already held by the tube.
//   IBCs:    IBCSubsets::Initialize (src/IBCSubsets.cpp:11-116) and
//            IBCMatrixManipulations::AddIBCFiniteDifference / AddIBCExtension
//            (src/IBCMatrixManipulations.cpp:12-251,424-463) as a patch:
//            moved stencil columns per tube row, extra IBC DOF rows whose E row
//            is the tricubic stencil at cp-bar (negated, + 2 g), identity rows.
// Per-node work runs in kernels (K6 IBC distance of every tube node, K7
// closest-point Jacobian + 3x3 eigen frames of every tube node, cp-bar and
// stencil weights); the host orders the small IBC subsets in the reference's
// BFS order and assembles the patch lists (K8).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <limits>
#include <unordered_map>

#include "eig3.h"
#include "opset.h"

namespace cpm {

template <class T>
static OpView<T> make_view(const cpm_opset_s *o, const T *w, const T *xval, const T *lval, const T *ldiag, const T *w_ord,
                           const T *pl_xval, const T *pe_w, const T *sp_w, const T *ov_w) {
    OpView<T> v;
    v.bv = o->tube->view();
    v.N = o->N;
    v.D = o->D;
    v.key = o->tube->key.p;
    v.base = o->base.p;
    v.w = w;
    v.flags = o->flags.p;
    v.patch = o->patch.p;
    v.p_emask = o->p_emask.p;
    v.p_eoff = o->p_eoff.p;
    v.p_lmask = o->p_lmask.p;
    v.p_loff = o->p_loff.p;
    v.moved = o->moved.p;
    v.p_xcol = o->p_xcol.p;
    v.p_xval = xval;
    v.lptr = o->lptr.p;
    v.lcol = o->lcol.p;
    v.lval = lval;
    v.ldiag = ldiag;
    // FDMatrices::BuildLaplacianMatrix: -2*dim and 1, then L /= dx*dx (src/FDMatrices.cpp:28-48)
    v.Ldiag = (T)(-6.0 / (o->dx * o->dx));
    v.Loff = (T)(1.0 / (o->dx * o->dx));
    v.nbr6 = o->nbr6.p;
    v.ord = o->ord.p;
    v.grp = o->grp.p;
    v.ident = o->ident.p;
    v.gcols = o->gcols.p;
    v.w_ord = w_ord;
    v.fl_ord = o->fl_ord.p;
    v.n_ord = o->n_ord;
    v.n_grp = o->n_grp;
    v.n_ident = o->n_ident;
    v.pl_row = o->pl_row.p;
    v.pl_off = o->pl_off.p;
    v.pl_xcol = o->pl_xcol.p;
    v.pl_neg = o->pl_neg.p;
    v.pl_xval = pl_xval;
    v.pe_new = o->pe_new.p;
    v.pe_old = o->pe_old.p;
    v.pe_w = pe_w;
    v.n_pl = o->n_pl;
    v.n_sp_rows = o->n_sp_rows;
    v.e32_bps = o->e32_bps;
    v.patch_bps = o->patch_bps;
    v.e64_bps = o->e64_bps;
    v.sp_ptr = o->n_sp_rows ? o->sp_ptr.p : nullptr;
    v.sp_rec = o->sp_rec.p;
    v.sp_w = sp_w;
    v.sp_rows = o->sp_rows.p;
    v.ov_ptr = o->ov_ptr.p;
    v.ov_col = o->ov_col.p;
    v.ov_w = ov_w;
    return v;
}

}  // namespace cpm

template <>
cpm::OpView<double> cpm_opset_s::view<double>() const {
    return cpm::make_view<double>(this, w.p, p_xval.p, lval.p, ldiag.p, w_ord.p, pl_xval.p, pe_w.p, sp_w.p, ov_w.p);
}
template <>
cpm::OpView<float> cpm_opset_s::view<float>() const {
    return cpm::make_view<float>(this, w32.p, p_xval32.p, lval32.p, ldiag32.p, w_ord32.p, pl_xval32.p, pe_w32.p, sp_w32.p, ov_w32.p);
}

namespace cpm {

// ---------------------------------------------------------------- host mirror of the tube tables
struct HostTube {
    std::vector<int32_t> bmap, bstart;
    std::vector<uint64_t> bmask;
    std::vector<uint32_t> key;
    std::vector<double> cp;
    int NB = 0, N1d = 0;
    double dx = 0, xstart = 0, radius = 0;
    int64_t N = 0;
    int load(const cpm_tube_s *t) {
        NB = t->g.NB;
        N1d = t->g.N1d;
        dx = t->g.dx;
        xstart = t->g.xstart;
        radius = t->g.radius;
        N = t->N;
        CPM_TRY(t->bmap.download(bmap, (size_t)NB * NB * NB));
        CPM_TRY(t->bstart.download(bstart, t->nbricks));
        CPM_TRY(t->bmask.download(bmask, t->nbricks));
        CPM_TRY(t->key.download(key, N));
        CPM_TRY(t->cp.download(cp, 3 * N));
        return 0;
    }
    int node(int i, int j, int k) const {
        if (i < 0 || j < 0 || k < 0 || i >= N1d || j >= N1d || k >= N1d) return -1;
        int r = bmap[((size_t)(i >> 2) * NB + (j >> 2)) * NB + (k >> 2)];
        if (r < 0) return -1;
        int l = ((i & 3) << 4) | ((j & 3) << 2) | (k & 3);
        uint64_t m = bmask[r];
        if (!((m >> l) & 1ull)) return -1;
        return bstart[r] + __builtin_popcountll(m & ((1ull << l) - 1ull));
    }
    // Node::neighbour(nbr), order +x,-x,+y,-y,+z,-z
    int nbr(int64_t q, int d) const {
        uint32_t kk = key[q];
        int i = unpack_i(kk) + (d == 0) - (d == 1), j = unpack_j(kk) + (d == 2) - (d == 3), k = unpack_k(kk) + (d == 4) - (d == 5);
        return node(i, j, k);
    }
    void x(int64_t q, double out[3]) const {
        uint32_t kk = key[q];
        out[0] = xstart + (double)unpack_i(kk) * dx;
        out[1] = xstart + (double)unpack_j(kk) * dx;
        out[2] = xstart + (double)unpack_k(kk) * dx;
    }
    // Tube::NearestTubeIndex (src/Tube.h:116-121)
    int64_t nearest(const double p[3]) const {
        int t[3];
        for (int d = 0; d < 3; ++d) t[d] = (int)std::round((p[d] - xstart) / dx);
        return node(t[0], t[1], t[2]);
    }
};

static inline double hdot(const double *a, const double *b) {
    double s = 0.0;
    for (int d = 0; d < 3; ++d) s += a[d] * b[d];
    return s;
}

// ---------------------------------------------------------------- K7: Jcp frames of the whole tube
// Dc_c cp_r per node (FDMatrices::BuildGradientMatrices, src/FDMatrices.cpp:66-92).
__global__ void k_cp_gradients(BrickView bv, int64_t N, const uint32_t *__restrict__ key, const double *__restrict__ cp, double dx,
                               double *__restrict__ g) {
    int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (q >= N) return;
    uint32_t kk = key[q];
    int i = unpack_i(kk), j = unpack_j(kk), k = unpack_k(kk);
    const double cplus = 0.5 / dx, cminus = -0.5 / dx;
    for (int c = 0; c < 3; ++c) {
        int np = node_at(bv, i + (c == 0), j + (c == 1), k + (c == 2));
        int nm = node_at(bv, i - (c == 0), j - (c == 1), k - (c == 2));
        for (int r = 0; r < 3; ++r) {
            double s = 0.0;
            if (np >= 0) s += cplus * cp[3 * (int64_t)np + r];
            if (nm >= 0) s += cminus * cp[3 * (int64_t)nm + r];
            g[9 * q + 3 * r + c] = s;
        }
    }
}

// (E g) for a 9-wide row-major vector on the plain tube stencil.
__global__ void k_extend9(OpView<double> op, const double *__restrict__ g, double *__restrict__ J) {
    int64_t gid = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    int64_t r = gid / 9;
    int s = (int)(gid % 9);
    if (r >= op.N) return;
    J[r * 9 + s] = e_row<double, 9>(op, r, s, g);
}

// Eigenvector of the smallest eigenvalue of 0.5 (J + J^T): the unoriented surface normal
// (IBCSubset::ComputeFrameBasedDirections, src/IBCSubset.cpp:192-228).
__global__ void k_jcp_normals(int64_t N, const double *__restrict__ J, double *__restrict__ nrm) {
    int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (q >= N) return;
    double A[3][3];
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) A[r][c] = 0.5 * (J[9 * q + 3 * r + c] + J[9 * q + 3 * c + r]);
    Eig3 e = sym_eig3(A);
    for (int r = 0; r < 3; ++r) nrm[3 * q + r] = e.vec[r][0];
}

__global__ void k_node_coords(int64_t N, const uint32_t *__restrict__ key, double xstart, double dx, double *__restrict__ x) {
    int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (q >= N) return;
    uint32_t kk = key[q];
    x[3 * q] = xstart + (double)unpack_i(kk) * dx;
    x[3 * q + 1] = xstart + (double)unpack_j(kk) * dx;
    x[3 * q + 2] = xstart + (double)unpack_k(kk) * dx;
}

// ---------------------------------------------------------------- host helpers for the IBC subsets

struct QueryRows {  // base points + weights of query points (computed on the device)
    std::vector<uint32_t> base;
    std::vector<double> w;
};

static int query_weights(const cpm_tube_s *t, const std::vector<double> &pts, QueryRows &out) {
    int64_t n = (int64_t)pts.size() / 3;
    out.base.clear();
    out.w.clear();
    if (n == 0) return 0;
    DBuf<double> dp, dw;
    DBuf<uint32_t> db;
    DBuf<int32_t> err;
    CPM_TRY(dp.upload(pts));
    CPM_TRY(db.alloc(n));
    CPM_TRY(dw.alloc(12 * n));
    CPM_TRY(err.alloc(1));
    CPM_TRY(err.zero());
    CPM_TRY(interp_weights_dev(t, n, dp.p, db.p, dw.p, err.p));
    std::vector<int32_t> he;
    CPM_TRY(err.download(he, 1));
    if (he[0]) return fail(CPM_ERR_BASEPOINT_OUTSIDE_TUBE, "Tube::ComputeBasePoints - Interpolation base point is not within the tube");
    CPM_TRY(db.download(out.base, n));
    CPM_TRY(dw.download(out.w, 12 * n));
    return 0;
}

// Stencil node of sidx = 16 i + 4 j + k and its E value w2[k]*w1[j]*w0[i]
// (src/Interpolation.cpp:99).
static inline void stencil_entry(const HostTube &ht, const QueryRows &qr, int64_t q, int sidx, int &col, double &val) {
    int i = sidx >> 4, j = (sidx >> 2) & 3, k = sidx & 3;
    uint32_t b = qr.base[q];
    col = ht.node(unpack_i(b) + i, unpack_j(b) + j, unpack_k(b) + k);
    const double *w = &qr.w[12 * q];
    val = w[8 + k] * w[4 + j] * w[i];
}

struct IBCData {
    cpm_surface_desc desc;
    std::vector<int64_t> tag_set;       // tube indices, BFS order
    std::vector<int64_t> tag_sub;       // N -> tagging index or -1
    std::vector<double> tag_cpc, tag_dist, tag_cpdiff, tag_dir, tag_binormal;
    std::vector<uint8_t> tag_bdy;
    std::vector<int64_t> dof_of_tag;    // tagging index -> dof index or -1
    std::vector<int64_t> dof_set;       // tube indices
    std::vector<int64_t> dof_sub;       // N -> dof index or -1
    std::vector<double> dof_cp, dof_cpbar, dof_dir, dof_cpdiff;
    QueryRows dof_rows;                 // E_ibc stencils (at cp or cp-bar)
    std::vector<uint8_t> side;          // per DOF: which side of the curve (1 or 2; 1 when not oriented)
    std::vector<int64_t> dir_sub;       // per DOF: index among the Dirichlet DOFs, or -1
    int64_t n_dir = 0;                  // Dirichlet DOFs of a 2nd-order IBC (value rows)
    bool order2 = false;
    bool has_dir2 = false;              // 2nd order with a Dirichlet side (IBCSubsets::TotalDOFs)
    // boundary type of DOF i's side (IBCMetaData::boundary_type[which_side - 1])
    int bc_type(size_t i) const { return desc.boundary_type[(side[i] == 2) ? 1 : 0]; }
    bool dof_dirichlet(size_t i) const { return bc_type(i) == 0; }
};

// Geometry::InterpolateUnorientedVectorFromNeighbours (src/Geometry.cpp:146-188).
static void interp_from_neighbours(const HostTube &ht, std::vector<double> &vec, const std::vector<int64_t> &set,
                                   const std::vector<int64_t> &sub, size_t i, double tol) {
    double acc[3] = {0, 0, 0}, first[3] = {0, 0, 0};
    size_t num = 0;
    for (int d = 0; d < 6; ++d) {
        int nb = ht.nbr(set[i], d);
        if (nb < 0) continue;
        int64_t s = sub[nb];
        if (s < 0) continue;
        const double *v = &vec[3 * s];
        if (std::sqrt(hdot(v, v)) >= tol) {
            if (num == 0)
                for (int k = 0; k < 3; ++k) first[k] = v[k];
            double sg = hdot(first, v) > 0 ? 1.0 : -1.0;
            for (int k = 0; k < 3; ++k) acc[k] = (sg > 0) ? acc[k] + v[k] : acc[k] - v[k];
            ++num;
        }
    }
    if (num > 0)
        for (int k = 0; k < 3; ++k) vec[3 * i + k] = acc[k] / (double)num;
}

// Geometry::InterpolateUnorientedVectors + ApplyInterpolationToUnorientedVectors
// (src/Geometry.cpp:205-266), normalised; columns restricted by colmap (-1 drops).
static std::vector<double> interp_unoriented(const HostTube &ht, const QueryRows &qr, const std::vector<double> &vecs,
                                             const std::vector<int64_t> *colmap) {
    size_t n = qr.base.size();
    std::vector<double> out(3 * n, 0.0);
    std::vector<std::pair<int64_t, double>> ent;
    for (size_t q = 0; q < n; ++q) {
        ent.clear();
        for (int s = 0; s < 64; ++s) {
            int col;
            double val;
            stencil_entry(ht, qr, (int64_t)q, s, col, val);
            if (col < 0) continue;
            int64_t c = colmap ? (*colmap)[col] : col;
            if (c >= 0) ent.push_back({c, val});
        }
        std::sort(ent.begin(), ent.end(), [](const std::pair<int64_t, double> &a, const std::pair<int64_t, double> &b) {
            return a.first < b.first;
        });
        double first[3] = {0, 0, 0}, acc[3] = {0, 0, 0};
        for (size_t e = 0; e < ent.size(); ++e) {
            const double *v = &vecs[3 * ent[e].first];
            if (e == 0)
                for (int k = 0; k < 3; ++k) first[k] = v[k];
            bool plus = hdot(first, v) > 0.0;
            for (int k = 0; k < 3; ++k) acc[k] = plus ? acc[k] + ent[e].second * v[k] : acc[k] - ent[e].second * v[k];
        }
        double nn = std::sqrt(hdot(acc, acc));
        for (int k = 0; k < 3; ++k) out[3 * q + k] = (nn > 0.0) ? acc[k] / nn : 0.0;
    }
    return out;
}

// ---------------------------------------------------------------- IBC frames on the device
// ComputeFrameBasedDirections (src/IBCSubset.cpp:190-268) for a tagging subset:
// the surface normals interpolated at the IBC closest points as
// Geometry::InterpolateUnorientedVectors + ApplyInterpolationToUnorientedVectors
// (src/Geometry.cpp:205-266; the arithmetic of interp_unoriented above, in the
// same order), and the frames of Geometry::EigenDecompositionOfJcp restricted to
// the subset (src/Geometry.cpp:27-69: Dc and E on the subset, J = E (Dc_c cp_r),
// eigen-frames of 0.5 (J + J^T)).

__device__ inline double ddot3(const double *a, const double *b) {
    double s = 0.0;
    for (int d = 0; d < 3; ++d) s += a[d] * b[d];
    return s;
}

// Dc_c cp_r restricted to the subset: g[9 i + 3 r + c] per tagging index i
__global__ void k_subset_grad(BrickView bv, int64_t nt, const uint32_t *__restrict__ key, const int32_t *__restrict__ tag_set,
                              const int32_t *__restrict__ tag_sub, const double *__restrict__ tag_cpc, double dx,
                              double *__restrict__ g) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= nt) return;
    const double cplus = 0.5 / dx, cminus = -0.5 / dx;
    const uint32_t kk = key[tag_set[i]];
    const int a[3] = {unpack_i(kk), unpack_j(kk), unpack_k(kk)};
    for (int c = 0; c < 3; ++c) {
        int pp[3] = {a[0], a[1], a[2]}, mm[3] = {a[0], a[1], a[2]};
        pp[c] += 1;
        mm[c] -= 1;
        const int np = node_at(bv, pp[0], pp[1], pp[2]), nm = node_at(bv, mm[0], mm[1], mm[2]);
        const int32_t sp = np >= 0 ? tag_sub[np] : -1, sm = nm >= 0 ? tag_sub[nm] : -1;
        for (int r = 0; r < 3; ++r) {
            double s = 0.0;
            if (sp >= 0) s += cplus * tag_cpc[3 * (int64_t)sp + r];
            if (sm >= 0) s += cminus * tag_cpc[3 * (int64_t)sm + r];
            g[9 * i + 3 * r + c] = s;
        }
    }
}

// per tagging index: the unoriented surface normal interpolated at its IBC
// closest point (stencil entries in ascending column order, each signed to the
// first), the symmetrised J = E (Dc cp) and its eigen-frame, then the direction
// and binormal
__global__ void k_tag_frames(BrickView bv, int64_t nt, const uint32_t *__restrict__ qbase, const double *__restrict__ qw,
                             const int32_t *__restrict__ tag_sub, const double *__restrict__ g,
                             const double *__restrict__ normals, const double *__restrict__ tag_cpdiff,
                             double *__restrict__ tag_dir, double *__restrict__ tag_binormal) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= nt) return;
    const uint32_t b = qbase[i];
    const int bi = unpack_i(b), bj = unpack_j(b), bk = unpack_k(b);
    const double *w = qw + 12 * i;
    // the stencil's bricks in rank order: nodes ascend with the rank, then with l
    int rk[8], bx[8], by[8], bz[8], nbk = 0;
    const int X0 = bi >> 2, Y0 = bj >> 2, Z0 = bk >> 2;
    const int nx = ((bi + 3) >> 2) - X0 + 1, ny = ((bj + 3) >> 2) - Y0 + 1, nz = ((bk + 3) >> 2) - Z0 + 1;
    for (int ox = 0; ox < nx; ++ox)
        for (int oy = 0; oy < ny; ++oy)
            for (int oz = 0; oz < nz; ++oz) {
                const int X = X0 + ox, Y = Y0 + oy, Z = Z0 + oz;
                if (X >= bv.NB || Y >= bv.NB || Z >= bv.NB) continue;
                const int r = bv.bmap[((size_t)X * bv.NB + Y) * bv.NB + Z];
                if (r < 0) continue;
                int p = nbk++;
                while (p > 0 && rk[p - 1] > r) {
                    rk[p] = rk[p - 1];
                    bx[p] = bx[p - 1];
                    by[p] = by[p - 1];
                    bz[p] = bz[p - 1];
                    --p;
                }
                rk[p] = r;
                bx[p] = X;
                by[p] = Y;
                bz[p] = Z;
            }
    double first[3] = {0, 0, 0}, acc[3] = {0, 0, 0};
    bool have = false;
    for (int e = 0; e < nbk; ++e) {
        const uint64_t m = bv.bmask[rk[e]];
        const int st = bv.bstart[rk[e]];
        for (int l = 0; l < 64; ++l) {
            if (!((m >> l) & 1ull)) continue;
            const int si = 4 * bx[e] + (l >> 4) - bi, sj = 4 * by[e] + ((l >> 2) & 3) - bj, sk = 4 * bz[e] + (l & 3) - bk;
            if (si < 0 || si > 3 || sj < 0 || sj > 3 || sk < 0 || sk > 3) continue;
            const int col = st + __popcll(m & ((1ull << l) - 1ull));
            const double val = w[8 + sk] * w[4 + sj] * w[si];
            const double *v = normals + 3 * (int64_t)col;
            if (!have) {
                for (int k = 0; k < 3; ++k) first[k] = v[k];
                have = true;
            }
            const bool plus = ddot3(first, v) > 0.0;
            for (int k = 0; k < 3; ++k) acc[k] = plus ? acc[k] + val * v[k] : acc[k] - val * v[k];
        }
    }
    double n[3];
    const double nn = sqrt(ddot3(acc, acc));
    for (int k = 0; k < 3; ++k) n[k] = (nn > 0.0) ? acc[k] / nn : 0.0;
    // J over the stencil in s order, restricted to the subset
    double J[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    for (int s = 0; s < 64; ++s) {
        const int si = s >> 4, sj = (s >> 2) & 3, sk = s & 3;
        const int col = node_at(bv, bi + si, bj + sj, bk + sk);
        if (col < 0) continue;
        const int32_t c = tag_sub[col];
        if (c < 0) continue;
        const double val = w[8 + sk] * w[4 + sj] * w[si];
        for (int t = 0; t < 9; ++t) J[t] += val * g[9 * (int64_t)c + t];
    }
    double A[3][3];
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) A[r][c] = 0.5 * (J[3 * r + c] + J[3 * c + r]);
    const Eig3 eg = sym_eig3(A);
    const double *cd = tag_cpdiff + 3 * i;
    double *dir = tag_dir + 3 * i, *bn = tag_binormal + 3 * i;
    if (fabs(eg.val[2]) < 1e-8) {
        const double dn = ddot3(n, cd);
        for (int k = 0; k < 3; ++k) {
            dir[k] = cd[k] - dn * n[k];
            bn[k] = 0.0;
        }
    } else {
        const double tg[3] = {eg.vec[0][2], eg.vec[1][2], eg.vec[2][2]};
        const double bb[3] = {tg[1] * n[2] - tg[2] * n[1], tg[2] * n[0] - tg[0] * n[2], tg[0] * n[1] - tg[1] * n[0]};
        const double bc = ddot3(bb, cd);
        for (int k = 0; k < 3; ++k) {
            bn[k] = bb[k];
            dir[k] = bc * bb[k];
        }
    }
}

// the frame directions of an IBC's tagging subset, computed on the device from
// the tube's unoriented normals (3 N, device)
static int tag_frames_dev(cpm_tube_s *t, IBCData &ib, const double *normals_dev) {
    const int64_t nt = (int64_t)ib.tag_set.size();
    ib.tag_dir.assign(3 * nt, 0.0);
    ib.tag_binormal.assign(3 * nt, 0.0);
    if (nt == 0) return 0;
    std::vector<int32_t> set(ib.tag_set.begin(), ib.tag_set.end()), sub(ib.tag_sub.begin(), ib.tag_sub.end());
    DBuf<int32_t> dset, dsub, derr;
    DBuf<double> dcpc, dcd, dg, ddir, dbn, dw;
    DBuf<uint32_t> db;
    CPM_TRY(dset.upload(set));
    CPM_TRY(dsub.upload(sub));
    CPM_TRY(dcpc.upload(ib.tag_cpc));
    CPM_TRY(dcd.upload(ib.tag_cpdiff));
    CPM_TRY(db.alloc(nt));
    CPM_TRY(dw.alloc(12 * nt));
    CPM_TRY(derr.alloc(1));
    CPM_TRY(derr.zero());
    CPM_TRY(interp_weights_dev(t, nt, dcpc.p, db.p, dw.p, derr.p));
    std::vector<int32_t> he;
    CPM_TRY(derr.download(he, 1));
    if (he[0]) return fail(CPM_ERR_BASEPOINT_OUTSIDE_TUBE, "Tube::ComputeBasePoints - Interpolation base point is not within the tube");
    CPM_TRY(dg.alloc(9 * nt));
    CPM_TRY(ddir.alloc(3 * nt));
    CPM_TRY(dbn.alloc(3 * nt));
    const unsigned nb = (unsigned)((nt + 127) / 128);
    k_subset_grad<<<nb, 128, 0, stream()>>>(t->view(), nt, t->key.p, dset.p, dsub.p, dcpc.p, t->g.dx, dg.p);
    k_tag_frames<<<nb, 128, 0, stream()>>>(t->view(), nt, db.p, dw.p, dsub.p, dg.p, normals_dev, dcd.p, ddir.p, dbn.p);
    CPM_CUDA_TRY(cudaGetLastError());
    CPM_TRY(ddir.download(ib.tag_dir, 3 * nt));
    CPM_TRY(dbn.download(ib.tag_binormal, 3 * nt));
    return 0;
}

// Geometry::UnorientedSurfaceNormals (src/Geometry.cpp:101-126) with its defaults
// (normalised, zero_tol 1e-15): x - cp, interpolated from the neighbours where it
// vanishes, then normalised (zero below the tolerance, src/VectorMath.cpp:40-56).
// The frames of an IBC with use_Jcp_surface_normals off use these.
static std::vector<double> unoriented_normals(const HostTube &ht) {
    const int64_t N = ht.N;
    std::vector<double> n(3 * N);
    for (int64_t q = 0; q < N; ++q) {
        double x[3];
        ht.x(q, x);
        for (int k = 0; k < 3; ++k) n[3 * q + k] = x[k] - ht.cp[3 * q + k];
    }
    std::vector<int64_t> ident(N);
    for (int64_t q = 0; q < N; ++q) ident[q] = q;
    const double zero_tol = 1e-15;
    for (int64_t q = 0; q < N; ++q)
        if (std::sqrt(hdot(&n[3 * q], &n[3 * q])) < zero_tol) interp_from_neighbours(ht, n, ident, ident, (size_t)q, zero_tol);
    for (int64_t q = 0; q < N; ++q) {
        const double nn = std::sqrt(hdot(&n[3 * q], &n[3 * q]));
        for (int k = 0; k < 3; ++k) n[3 * q + k] = nn > zero_tol ? n[3 * q + k] / nn : 0.0;
    }
    return n;
}

// First parameterisation point of an IBC (IBCSubset::FindStartingPoint uses xp()[0]):
// paramCircle3D vertex 0 (src/Surface.cpp:1883-1904), the point itself, or vertex 0.
// the unit basis t1, t2 of a circle's plane (ComputeOrthogonalBasis + Normalize)
static void circle_basis(const double *p, double t1[3], double t2[3]) {
    double n[3] = {p[4], p[5], p[6]};
    if (std::fabs(n[0]) > std::fabs(n[1])) {
        t1[0] = -n[2]; t1[1] = 0; t1[2] = n[0];
    } else {
        t1[0] = 0; t1[1] = n[2]; t1[2] = -n[1];
    }
    t2[0] = n[1] * t1[2] - n[2] * t1[1];
    t2[1] = n[2] * t1[0] - n[0] * t1[2];
    t2[2] = n[0] * t1[1] - n[1] * t1[0];
    double n1 = std::sqrt(hdot(t1, t1)), n2 = std::sqrt(hdot(t2, t2));
    for (int k = 0; k < 3; ++k) {
        t1[k] = n1 > 0 ? t1[k] / n1 : 0;
        t2[k] = n2 > 0 ? t2[k] / n2 : 0;
    }
}

// plot point i of a Circle3D (Surface::paramCircle3D, src/Surface.cpp:1883-1904):
// theta_i = i 2 pi / (Np - 1), Np = 100
constexpr int64_t CIRCLE_NP = 100;
static void circle_point(const double *p, int64_t i, double out[3]) {
    double t1[3], t2[3];
    circle_basis(p, t1, t2);
    const double th = (double)i * (2.0 * M_PI / (double)(CIRCLE_NP - 1));
    const double c = std::cos(th), sn = std::sin(th);
    for (int k = 0; k < 3; ++k) out[k] = p[1 + k] + p[0] * (c * t1[k] + sn * t2[k]);
}

static void ibc_xp0(const cpm_surface_desc &d, const std::vector<double> &verts, double out[3]) {
    if (d.kind == CPM_CIRCLE3D) {
        circle_point(d.params, 0, out);
    } else if (d.kind == CPM_POINT) {
        for (int k = 0; k < 3; ++k) out[k] = d.params[k];
    } else {
        for (int k = 0; k < 3; ++k) out[k] = verts[k];
    }
}

// Caller-supplied closest points (cpm_opset_create_from_cp): a table from query
// points, matched by the exact bits of their three coordinates, to the closest
// point and distance the caller computed there.  Points the table lacks keep
// the device's own closest point.
struct CpTable {
    struct Key {
        uint64_t a, b, c;
        bool operator==(const Key &o) const { return a == o.a && b == o.b && c == o.c; }
    };
    struct Hash {
        size_t operator()(const Key &k) const {
            uint64_t h = k.a * 0x9E3779B97F4A7C15ull;
            h ^= k.b + 0x7F4A7C159E3779B9ull + (h << 6) + (h >> 2);
            h ^= k.c + 0x94D049BB133111EBull + (h << 6) + (h >> 2);
            return (size_t)h;
        }
    };
    std::unordered_map<Key, int64_t, Hash> index;
    std::vector<double> cp, dist;  // copies: an operator set keeps its tables for later evaluation queries
    static Key key(const double *x) {
        Key k;
        memcpy(&k.a, x, 8);
        memcpy(&k.b, x + 1, 8);
        memcpy(&k.c, x + 2, 8);
        return k;
    }
    void load(const cpm_cp_table *t) {
        index.clear();
        cp.clear();
        dist.clear();
        if (!t || t->n <= 0 || !t->x || !t->cp) return;
        cp.assign(t->cp, t->cp + 3 * t->n);
        if (t->dist) dist.assign(t->dist, t->dist + t->n);
        index.reserve((size_t)t->n);
        for (int64_t i = 0; i < t->n; ++i) index.emplace(key(t->x + 3 * i), i);
    }
    bool empty() const { return index.empty(); }
    // overrides cp_out (and dist_out when the table has distances) for a point it holds
    bool lookup(const double *x, double *cp_out, double *dist_out) const {
        auto it = index.find(key(x));
        if (it == index.end()) return false;
        for (int k = 0; k < 3; ++k) cp_out[k] = cp[3 * it->second + k];
        if (!dist.empty() && dist_out) *dist_out = dist[it->second];
        return true;
    }
};

struct CpOverrides {
    std::vector<CpTable> ibc;  // per IBC: its closest points at tube-node coordinates
    CpTable surface;           // the tube surface's closest points at the cp-bar projections
};

// ---------------------------------------------------------------- tagging walk on the device
// IBCSubset::ComputeSubsetNearIBC (src/IBCSubset.cpp:39-109): a breadth-first
// walk over tube neighbours from `start`, keeping the nodes with dist < lim, in
// the order a FIFO queue discovers them.  One thread block walks level by level:
// a node of the next level belongs to the smallest (frontier position p,
// neighbour d) that reaches it while it is unvisited (t = 6 p + d, by atomicMin),
// and the level's accepted nodes are compacted in increasing t, which is the
// queue's discovery order.  `start` begins unvisited, as in the reference, so
// it joins the subset if the walk reaches it again.  Every loop is bounded
// (each level visits new nodes; at most cap accepted); err = 1 if cap is hit.
constexpr int BFS_T = 1024;
__global__ void __launch_bounds__(BFS_T) k_tag_walk(BrickView bv, const uint32_t *__restrict__ key, int start,
                                                   const double *__restrict__ dist, double lim, uint8_t *__restrict__ visited,
                                                   int32_t *__restrict__ kmin, int32_t *__restrict__ front0,
                                                   int32_t *__restrict__ front1, int32_t *__restrict__ tag_set, int32_t cap,
                                                   int32_t *__restrict__ n_out, int *__restrict__ err) {
    __shared__ int32_t warp_sum[BFS_T / 32];
    __shared__ int32_t s_carry, s_F, s_nt;
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    if (tid == 0) {
        front0[0] = start;
        s_F = 1;
        s_nt = 0;
    }
    __syncthreads();
    int32_t *front = front0, *next = front1;
    for (int level = 0; level < cap + 1; ++level) {
        const int F = s_F;
        if (F == 0) break;
        const int T = 6 * F;
        for (int t = tid; t < T; t += BFS_T) {
            const uint32_t kk = key[front[t / 6]];
            const int d = t % 6;
            const int nb = node_at(bv, unpack_i(kk) + (d == 0) - (d == 1), unpack_j(kk) + (d == 2) - (d == 3),
                                   unpack_k(kk) + (d == 4) - (d == 5));
            if (nb >= 0 && !visited[nb]) atomicMin(&kmin[nb], t);
        }
        if (tid == 0) s_carry = 0;
        __syncthreads();
        for (int base = 0; base < T; base += BFS_T) {
            const int t = base + tid;
            int nb = -1, acc = 0;
            bool own = false;
            if (t < T) {
                const uint32_t kk = key[front[t / 6]];
                const int d = t % 6;
                nb = node_at(bv, unpack_i(kk) + (d == 0) - (d == 1), unpack_j(kk) + (d == 2) - (d == 3),
                             unpack_k(kk) + (d == 4) - (d == 5));
                own = nb >= 0 && !visited[nb] && kmin[nb] == t;
                acc = (own && dist[nb] < lim) ? 1 : 0;
            }
            // exclusive scan of acc over the block
            int x = acc;
            for (int o = 1; o < 32; o <<= 1) {
                const int y = __shfl_up_sync(0xffffffffu, x, o);
                if (lane >= o) x += y;
            }
            if (lane == 31) warp_sum[wid] = x;
            __syncthreads();
            if (wid == 0) {
                int w = warp_sum[lane];
                for (int o = 1; o < 32; o <<= 1) {
                    const int y = __shfl_up_sync(0xffffffffu, w, o);
                    if (lane >= o) w += y;
                }
                warp_sum[lane] = w;  // inclusive over warps
            }
            __syncthreads();
            const int before = (wid > 0 ? warp_sum[wid - 1] : 0) + x - acc;
            const int chunk = warp_sum[BFS_T / 32 - 1];
            const int carry = s_carry;
            if (acc) {
                const int pos = carry + before, slot = s_nt + pos;
                if (slot < cap && pos < cap) {
                    next[pos] = nb;
                    tag_set[slot] = nb;
                } else {
                    atomicOr(err, 1);
                }
            }
            if (own) {
                visited[nb] = 1;
                kmin[nb] = 0x7fffffff;
            }
            __syncthreads();
            if (tid == 0) s_carry = carry + chunk;
            __syncthreads();
        }
        if (tid == 0) {
            const int nF = s_carry;
            s_nt = min(cap, s_nt + nF);
            s_F = (*err) ? 0 : min(nF, cap);
        }
        __syncthreads();
        int32_t *tmp = front;
        front = next;
        next = tmp;
    }
    if (tid == 0) *n_out = s_nt;
}

// tag_cpc / tag_dist of the walked subset from the IBC closest points of all tube nodes
__global__ void k_tag_gather(int64_t nt, const int32_t *__restrict__ tag_set, const double *__restrict__ cp,
                             const double *__restrict__ dist, double *__restrict__ tag_cpc, double *__restrict__ tag_dist) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= nt) return;
    const int64_t q = tag_set[i];
    for (int k = 0; k < 3; ++k) tag_cpc[3 * i + k] = cp[3 * q + k];
    tag_dist[i] = dist[q];
}

__global__ void k_count_below(int64_t n, const double *__restrict__ v, double lim, unsigned long long *__restrict__ cnt) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const bool b = i < n && v[i] < lim;
    const unsigned m = __ballot_sync(0xffffffffu, b);
    if ((threadIdx.x & 31) == 0 && m) atomicAdd(cnt, (unsigned long long)__popc(m));
}

static int build_ibc_data(cpm_tube_s *t, const HostTube &ht, const cpm_surface_desc &desc, const double *normals_dev,
                          const DBuf<double> &xdev, const CpTable *cpt, const CpTable *surf_cpt,
                          IBCData &ib) {
    const int64_t N = ht.N;
    const double r = ht.radius;
    ib.desc = desc;
    ib.order2 = desc.boundary_order == 2;
    ib.has_dir2 = ib.order2 && (desc.boundary_type[0] == 0 || desc.boundary_type[1] == 0);
    // K6: IBC closest point + distance of every tube node (bounded at 2r for meshes)
    SurfaceObj s;
    CPM_TRY(surface_init(s, &desc, r));
    std::vector<double> verts;
    if (desc.kind == CPM_TRIANGULATION || desc.kind == CPM_POLYLINE) verts.assign(desc.verts, desc.verts + 3 * desc.nverts);
    DBuf<double> dcp, dd;
    CPM_TRY(dcp.alloc(3 * N));
    CPM_TRY(dd.alloc(N));
    CPM_TRY(closest_points_dev(s.params(), N, xdev.p, dcp.p, dd.p, 2.0 * r * (1.0 + 1e-12)));
    if (cpt && !cpt->empty()) {
        // the caller's closest points for the nodes its table holds (parity checks)
        std::vector<double> cpc, distc;
        CPM_TRY(dcp.download(cpc, 3 * N));
        CPM_TRY(dd.download(distc, N));
        for (int64_t q = 0; q < N; ++q) {
            double xq[3];
            ht.x(q, xq);
            cpt->lookup(xq, &cpc[3 * q], &distc[q]);
        }
        CPM_TRY(dcp.upload(cpc));
        CPM_TRY(dd.upload(distc));
    }
    // open polylines tag closest points at their end points (src/Surface.cpp:2614-2637)
    bool open_poly = false;
    if (desc.kind == CPM_POLYLINE && desc.nverts > 1) {
        const double *v0 = desc.verts, *vl = desc.verts + 3 * (desc.nverts - 1);
        bool same = v0[0] == vl[0] && v0[1] == vl[1] && v0[2] == vl[2];
        const int64_t *lastf = desc.prims + 2 * (desc.nprims - 1);
        open_poly = !(same || lastf[0] == 0 || lastf[1] == 0);
    }
    // IBCSubset::ComputeSubsetNearIBC (src/IBCSubset.cpp:39-109): BFS over tube
    // neighbours from the node nearest xp[0], keeping dist < 2r, in queue order.
    double xp0[3];
    ibc_xp0(desc, verts, xp0);
    int64_t start = ht.nearest(xp0);
    if (start < 0) return fail(CPM_ERR_INVALID_ARG, "IBC start point is not near the tube");
    {
        // the walk on the device (k_tag_walk), sized by the nodes within 2r
        DBuf<unsigned long long> dcnt;
        CPM_TRY(dcnt.alloc(1));
        CPM_TRY(dcnt.zero());
        k_count_below<<<(unsigned)((N + 255) / 256), 256, 0, stream()>>>(N, dd.p, 2.0 * r, dcnt.p);
        std::vector<unsigned long long> hc;
        CPM_TRY(dcnt.download(hc, 1));
        const int32_t cap = (int32_t)hc[0] + 1;
        DBuf<uint8_t> vis;
        DBuf<int32_t> kmin, f0, f1, dset, dn;
        DBuf<int> derr;
        CPM_TRY(vis.alloc(N));
        CPM_TRY(vis.zero());
        CPM_TRY(kmin.alloc(N));
        CPM_CUDA_TRY(cudaMemsetAsync(kmin.p, 0x7f, N * sizeof(int32_t), stream()));  // 0x7f7f7f7f > any 6 p + d
        CPM_TRY(f0.alloc(cap));
        CPM_TRY(f1.alloc(cap));
        CPM_TRY(dset.alloc(cap));
        CPM_TRY(dn.alloc(1));
        CPM_TRY(derr.alloc(1));
        CPM_TRY(derr.zero());
        k_tag_walk<<<1, BFS_T, 0, stream()>>>(t->view(), t->key.p, (int)start, dd.p, 2.0 * r, vis.p, kmin.p, f0.p, f1.p,
                                              dset.p, cap, dn.p, derr.p);
        CPM_CUDA_TRY(cudaGetLastError());
        std::vector<int32_t> hn, he, hs;
        CPM_TRY(derr.download(he, 1));
        if (he[0]) return fail(CPM_ERR_CUDA, "internal: the tagging walk outgrew its bound");
        CPM_TRY(dn.download(hn, 1));
        const int64_t ntw = hn[0];
        CPM_TRY(dset.download(hs, ntw));
        ib.tag_set.assign(hs.begin(), hs.end());
        ib.tag_sub.assign(N, -1);
        for (int64_t i = 0; i < ntw; ++i) ib.tag_sub[hs[i]] = i;
        DBuf<double> dtc, dtd;
        CPM_TRY(dtc.alloc(3 * std::max<int64_t>(1, ntw)));
        CPM_TRY(dtd.alloc(std::max<int64_t>(1, ntw)));
        if (ntw > 0) {
            k_tag_gather<<<(unsigned)((ntw + 255) / 256), 256, 0, stream()>>>(ntw, dset.p, dcp.p, dd.p, dtc.p, dtd.p);
            CPM_CUDA_TRY(cudaGetLastError());
        }
        CPM_TRY(dtc.download(ib.tag_cpc, 3 * ntw));
        CPM_TRY(dtd.download(ib.tag_dist, ntw));
    }
    const size_t nt = ib.tag_set.size();
    ib.tag_bdy.assign(nt, 0);
    for (size_t i = 0; i < nt; ++i) {
        if (open_poly) {
            const double *v0 = desc.verts, *vl = desc.verts + 3 * (desc.nverts - 1);
            double d0 = 0, d1 = 0;
            const double *cq = &ib.tag_cpc[3 * i];
            for (int k = 0; k < 3; ++k) {
                d0 += (v0[k] - cq[k]) * (v0[k] - cq[k]);
                d1 += (vl[k] - cq[k]) * (vl[k] - cq[k]);
            }
            if (std::sqrt(d0) < 1e-7)
                ib.tag_bdy[i] = 1;
            else if (std::sqrt(d1) < 1e-7)
                ib.tag_bdy[i] = 2;
        }
    }
    // ComputeCPdiff (src/IBCSubset.cpp:156-187) with the S-perp fix-up: cp_S(x) - cp_c,
    // or, at an open polyline's end points when use_cp_diff_directions is on,
    // cp_c(p) - cp_S(p) at the reflection p = 2 cp_c - x
    ib.tag_cpdiff.resize(3 * nt);
    for (size_t i = 0; i < nt; ++i) {
        int64_t q = ib.tag_set[i];
        for (int k = 0; k < 3; ++k) ib.tag_cpdiff[3 * i + k] = ht.cp[3 * q + k] - ib.tag_cpc[3 * i + k];
    }
    if (desc.use_cp_diff_directions) {
        std::vector<size_t> ends;
        std::vector<double> proj;
        for (size_t i = 0; i < nt; ++i)
            if (ib.tag_bdy[i] > 0) {
                double x[3];
                ht.x(ib.tag_set[i], x);
                ends.push_back(i);
                for (int k = 0; k < 3; ++k) proj.push_back(2.0 * ib.tag_cpc[3 * i + k] - x[k]);
            }
        if (!ends.empty()) {
            const int64_t ne = (int64_t)ends.size();
            DBuf<double> dp, dcs, dds, dcc, ddc;
            CPM_TRY(dp.upload(proj));
            CPM_TRY(dcs.alloc(3 * ne));
            CPM_TRY(dds.alloc(ne));
            CPM_TRY(dcc.alloc(3 * ne));
            CPM_TRY(ddc.alloc(ne));
            const double inf = std::numeric_limits<double>::infinity();
            CPM_TRY(closest_points_dev(t->surf.params(), ne, dp.p, dcs.p, dds.p, inf));
            CPM_TRY(closest_points_dev(s.params(), ne, dp.p, dcc.p, ddc.p, inf));
            std::vector<double> cps, cpc2;
            CPM_TRY(dcs.download(cps, 3 * ne));
            CPM_TRY(dcc.download(cpc2, 3 * ne));
            for (int64_t e = 0; e < ne; ++e)
                for (int k = 0; k < 3; ++k) ib.tag_cpdiff[3 * ends[e] + k] = cpc2[3 * e + k] - cps[3 * e + k];
        }
    }
    for (size_t i = 0; i < nt; ++i)
        if (std::sqrt(hdot(&ib.tag_cpdiff[3 * i], &ib.tag_cpdiff[3 * i])) < desc.on_ibc_tolerance)
            interp_from_neighbours(ht, ib.tag_cpdiff, ib.tag_set, ib.tag_sub, i, desc.on_ibc_tolerance);
    if (desc.use_cp_diff_directions) {
        // IBCSubset::ComputeSubset: the directions are cp_diff itself
        ib.tag_dir = ib.tag_cpdiff;
        ib.tag_binormal.assign(3 * nt, 0.0);
    } else {
        // ComputeFrameBasedDirections (src/IBCSubset.cpp:190-268), on the device
        CPM_TRY(tag_frames_dev(t, ib, normals_dev));
    }
    // IBCDOFSubset::ComputeDOFSubset (src/IBCDOFSubset.cpp:10-93)
    const double rad = desc.dof_radius_scale * r;
    ib.dof_sub.assign(N, -1);
    ib.dof_of_tag.assign(nt, -1);
    for (size_t i = 0; i < nt; ++i)
        if (ib.tag_dist[i] < rad) {
            ib.dof_of_tag[i] = (int64_t)ib.dof_set.size();
            ib.dof_sub[ib.tag_set[i]] = (int64_t)ib.dof_set.size();
            ib.dof_set.push_back(ib.tag_set[i]);
            for (int k = 0; k < 3; ++k) {
                ib.dof_cp.push_back(ib.tag_cpc[3 * i + k]);
                ib.dof_cpdiff.push_back(ib.tag_cpdiff[3 * i + k]);
                ib.dof_dir.push_back(ib.tag_dir[3 * i + k]);
            }
        }
    const size_t nd = ib.dof_set.size();
    // which_side (OrientSubset, src/IBCDOFSubset.cpp:128-227): a breadth-first walk
    // over the DOF subset from its first DOF off the curve, a neighbour takes the
    // other side when its direction points against the current DOF's; then the
    // sides are swapped if the DOF nearest point_on_side1 (among those 2 dx or
    // more from the curve, on the point's side of it) came out on side 1
    ib.side.assign(nd, 1);
    if (desc.is_oriented && nd > 0) {
        std::fill(ib.side.begin(), ib.side.end(), (uint8_t)0);
        size_t start = 0;
        for (size_t i = 0; i < nd; ++i)
            if (std::sqrt(hdot(&ib.dof_dir[3 * i], &ib.dof_dir[3 * i])) >= desc.on_ibc_tolerance) {
                start = i;
                break;
            }
        ib.side[start] = 1;
        std::vector<size_t> queue{start};
        std::vector<uint8_t> seen(nd, 0);
        for (size_t h = 0; h < queue.size(); ++h) {
            const size_t f = queue[h];
            if (seen[f]) continue;
            seen[f] = 1;
            for (int d = 0; d < 6; ++d) {
                const int nb = ht.nbr(ib.dof_set[f], d);
                if (nb < 0) continue;
                const int64_t ns = ib.dof_sub[nb];
                if (ns < 0) continue;
                if (ib.side[ns] == 0)
                    ib.side[ns] = hdot(&ib.dof_dir[3 * f], &ib.dof_dir[3 * ns]) < 0 ? (ib.side[f] == 1 ? 2 : 1) : ib.side[f];
                queue.push_back((size_t)ns);
            }
        }
        if (desc.has_point_on_side1) {
            const double *ps = desc.point_on_side1;
            DBuf<double> dps, dcpc, ddc;
            CPM_TRY(dps.upload(ps, 3));
            CPM_TRY(dcpc.alloc(3));
            CPM_TRY(ddc.alloc(1));
            CPM_TRY(closest_points_dev(s.params(), 1, dps.p, dcpc.p, ddc.p, std::numeric_limits<double>::infinity()));
            std::vector<double> cpc_ps;
            CPM_TRY(dcpc.download(cpc_ps, 3));
            const double cpd[3] = {ps[0] - cpc_ps[0], ps[1] - cpc_ps[1], ps[2] - cpc_ps[2]};
            size_t nearest = 0;
            double best = std::numeric_limits<double>::max();
            for (size_t i = 0; i < nd; ++i) {
                double xi[3];
                ht.x(ib.dof_set[i], xi);
                double dd = 0.0;
                for (int k = 0; k < 3; ++k) dd += (ps[k] - xi[k]) * (ps[k] - xi[k]);
                dd = std::sqrt(dd);
                const double *cd = &ib.dof_cpdiff[3 * i];
                if (dd < best && std::sqrt(hdot(cd, cd)) >= 2.0 * ht.dx && hdot(cpd, cd) > 0) {
                    best = dd;
                    nearest = i;
                }
            }
            if (ib.side[nearest] == 1)
                for (auto &w : ib.side) w = (w == 1) ? 2 : (w == 2 ? 1 : w);
        }
        // a DOF the walk did not reach (a DOF subset in pieces) keeps side 1
        for (auto &w : ib.side)
            if (w == 0) w = 1;
    }
    // the Dirichlet DOFs of a 2nd-order IBC, in DOF order (their value rows)
    ib.dir_sub.assign(nd, -1);
    ib.n_dir = 0;
    if (ib.has_dir2)
        for (size_t i = 0; i < nd; ++i)
            if (ib.dof_dirichlet(i)) ib.dir_sub[i] = ib.n_dir++;
    if (ib.order2) {
        // cp-bar = cp_S(2 cp_c - x)  (src/IBCDOFSubset.cpp:63-73)
        std::vector<double> proj(3 * nd);
        for (size_t i = 0; i < nd; ++i) {
            double x[3];
            ht.x(ib.dof_set[i], x);
            for (int k = 0; k < 3; ++k) proj[3 * i + k] = 2.0 * ib.dof_cp[3 * i + k] - x[k];
        }
        DBuf<double> dp, dc, ddist;
        CPM_TRY(dp.upload(proj));
        CPM_TRY(dc.alloc(3 * nd));
        CPM_TRY(ddist.alloc(nd));
        CPM_TRY(closest_points_dev(t->surf.params(), (int64_t)nd, dp.p, dc.p, ddist.p, 4.0 * r));
        CPM_TRY(dc.download(ib.dof_cpbar, 3 * nd));
        if (surf_cpt && !surf_cpt->empty())
            for (size_t i = 0; i < nd; ++i) surf_cpt->lookup(&proj[3 * i], &ib.dof_cpbar[3 * i], nullptr);
        CPM_TRY(query_weights(t, ib.dof_cpbar, ib.dof_rows));
    } else {
        CPM_TRY(query_weights(t, ib.dof_cp, ib.dof_rows));
    }
    return 0;
}

// IBCDOFSubset::which_side as the reference hands it to the boundary-value
// function: the side of an oriented IBC's DOF, 0 when the IBC is not oriented
static inline int32_t desc_side(const IBCData &ib, size_t i) { return ib.desc.is_oriented ? (int32_t)ib.side[i] : 0; }

// tag of the stencil entry (row director dir_r, column node col) for one IBC
// (TagStencils, src/IBCMatrixManipulations.cpp:424-463).
static inline bool tagged(const IBCData &ib, const double *dir_r, int col, double flip) {
    int64_t sp = ib.tag_sub[col];
    if (sp < 0 || ib.tag_bdy[sp] != 0) return false;
    return flip * hdot(dir_r, &ib.tag_dir[3 * sp]) < 0.0;
}

// ---------------------------------------------------------------- TagStencils on the device
// One IBC's tagging as the device kernels read it.
struct IbcTagDev {
    const int32_t *tag_sub;  // N: tagging index or -1
    const uint8_t *tag_bdy;  // per tagging index: 0, or 1 / 2 at an open polyline's end points
    const double *tag_dir;   // 3 per tagging index
    const int32_t *dof_sub;  // N: DOF index or -1
    int64_t col_start;
};

// tagged() on the device: the same products and sums, in the same order
__device__ inline bool tagged_dev(const IbcTagDev &ib, const double *dir_r, int col, double flip) {
    const int32_t sp = ib.tag_sub[col];
    if (sp < 0 || ib.tag_bdy[sp] != 0) return false;
    const double *d = ib.tag_dir + 3 * (int64_t)sp;
    double s = 0.0;
    for (int k = 0; k < 3; ++k) s += dir_r[k] * d[k];
    return flip * s < 0.0;
}

// the IBC columns a tube row's entry (column col) moves to: one copy of the
// entry for every IBC whose tag crosses it and whose DOF subset holds col
// (MoveToIBCColumns, src/IBCMatrixManipulations.cpp:189-216), in IBC order.
// Returns their count; the first target in *first, the others in xout.
__device__ inline int tube_entry_targets(const IbcTagDev *ibs, int n_ibc, int64_t q, int col, int64_t *first,
                                         int32_t *xout) {
    int hits = 0;
    if (col < 0) return 0;
    for (int c = 0; c < n_ibc; ++c) {
        const int32_t tq = ibs[c].tag_sub[q];
        if (tq < 0) continue;
        if (tagged_dev(ibs[c], ibs[c].tag_dir + 3 * (int64_t)tq, col, 1.0) && ibs[c].dof_sub[col] >= 0) {
            const int64_t tgt = ibs[c].col_start + ibs[c].dof_sub[col];
            if (hits == 0)
                *first = tgt;
            else if (xout)
                xout[hits - 1] = (int32_t)tgt;
            ++hits;
        }
    }
    return hits;
}

// tube row q's moved E stencil entries (bit s = 16 i + 4 j + k) and L neighbours
// (bit d, order +x -x +y -y +z -z) with their counts, and the number of extra
// targets of entries that move to more than one IBC (xcount[2q]: E, [2q+1]: L).
// With moved != null instead the targets: first targets from moved[off[q]], E
// entries in s order then L entries in d order; extra targets from xcol[xoff[q]]
// in the same order, each with its s or d in xsd.
__global__ void k_tube_moves(BrickView bv, int64_t N, const uint32_t *__restrict__ key, const uint32_t *__restrict__ base,
                             const IbcTagDev *__restrict__ ibs, int n_ibc, uint64_t *__restrict__ emask,
                             uint8_t *__restrict__ lmask, int32_t *__restrict__ count, int32_t *__restrict__ xcount,
                             const int32_t *__restrict__ off, int32_t *__restrict__ moved, const int32_t *__restrict__ xoff,
                             int32_t *__restrict__ xcol, int32_t *__restrict__ xsd) {
    const int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (q >= N) return;
    bool any = false;
    for (int c = 0; c < n_ibc && !any; ++c) any = ibs[c].tag_sub[q] >= 0;
    uint64_t em = 0;
    uint8_t lm = 0;
    int cnt = 0, xe = 0, xl = 0;
    int32_t *out = moved ? moved + off[q] : nullptr;
    int32_t *xo = (moved && xcol) ? xcol + xoff[q] : nullptr;
    int32_t *xs = (moved && xcol) ? xsd + xoff[q] : nullptr;
    if (any) {
        const uint32_t b = base[q];
        const int bi = unpack_i(b), bj = unpack_j(b), bk = unpack_k(b);
        for (int s = 0; s < 64; ++s) {
            const int col = node_at(bv, bi + (s >> 4), bj + ((s >> 2) & 3), bk + (s & 3));
            int64_t tgt = -1;
            const int h = tube_entry_targets(ibs, n_ibc, q, col, &tgt, xo ? xo + xe : nullptr);
            if (h > 0) {
                em |= 1ull << s;
                if (out) out[cnt] = (int32_t)tgt;
                ++cnt;
                if (xs)
                    for (int e = 0; e < h - 1; ++e) xs[xe + e] = s;
                xe += h - 1;
            }
        }
        const uint32_t kk = key[q];
        const int i = unpack_i(kk), j = unpack_j(kk), k = unpack_k(kk);
        for (int d = 0; d < 6; ++d) {
            const int col = node_at(bv, i + (d == 0) - (d == 1), j + (d == 2) - (d == 3), k + (d == 4) - (d == 5));
            int64_t tgt = -1;
            const int h = tube_entry_targets(ibs, n_ibc, q, col, &tgt, xo ? xo + xe + xl : nullptr);
            if (h > 0) {
                lm |= (uint8_t)(1u << d);
                if (out) out[cnt] = (int32_t)tgt;
                ++cnt;
                if (xs)
                    for (int e = 0; e < h - 1; ++e) xs[xe + xl + e] = d;
                xl += h - 1;
            }
        }
    }
    if (!moved) {
        emask[q] = em;
        lmask[q] = lm;
        count[q] = cnt;
        xcount[2 * q] = xe;
        xcount[2 * q + 1] = xl;
    }
}

// an IBC's DOF rows (AddExtensionIBCRows, src/IBCMatrixManipulations.cpp:118-186;
// AddFiniteDifferenceIBCRows, :219-251): per DOF i, the E_ibc stencil entries
// (at dbase[i], in s order) tagged against the DOF's direction with flip -1 that
// move to a DOF column, and the six L columns (-1: dropped): across the curve
// the tube node itself, same side and in the DOF subset that DOF's column.
// With moved != null the E targets from moved[off[i]] instead.
__global__ void k_dof_moves(BrickView bv, int64_t nd, const uint32_t *__restrict__ key, const int32_t *__restrict__ dof_set,
                            const uint32_t *__restrict__ dbase, const double *__restrict__ dof_dir, IbcTagDev ib,
                            uint64_t *__restrict__ emask, int32_t *__restrict__ count, int32_t *__restrict__ lcols,
                            const int32_t *__restrict__ off, int32_t *__restrict__ moved) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= nd) return;
    const uint32_t b = dbase[i];
    const int bi = unpack_i(b), bj = unpack_j(b), bk = unpack_k(b);
    uint64_t em = 0;
    int cnt = 0;
    for (int s = 0; s < 64; ++s) {
        const int col = node_at(bv, bi + (s >> 4), bj + ((s >> 2) & 3), bk + (s & 3));
        if (col >= 0 && tagged_dev(ib, dof_dir + 3 * i, col, -1.0) && ib.dof_sub[col] >= 0) {
            em |= 1ull << s;
            if (moved) moved[off[i] + cnt] = (int32_t)(ib.col_start + ib.dof_sub[col]);
            ++cnt;
        }
    }
    if (moved) return;
    emask[i] = em;
    count[i] = cnt;
    const int node = dof_set[i];
    const uint32_t kk = key[node];
    const int x = unpack_i(kk), y = unpack_j(kk), z = unpack_k(kk);
    const int32_t tq = ib.tag_sub[node];
    for (int d = 0; d < 6; ++d) {
        const int col = node_at(bv, x + (d == 0) - (d == 1), y + (d == 2) - (d == 3), z + (d == 4) - (d == 5));
        int32_t lc = -1;
        if (col >= 0) {
            if (tq >= 0 && tagged_dev(ib, ib.tag_dir + 3 * (int64_t)tq, col, 1.0))
                lc = col;
            else if (ib.dof_sub[col] >= 0)
                lc = (int32_t)(ib.col_start + ib.dof_sub[col]);
        }
        lcols[6 * i + d] = lc;
    }
}

static int build_base(cpm_opset_s *o) {
    cpm_tube_s *t = o->tube;
    o->N = t->N;
    o->D = t->N;
    o->dx = t->g.dx;
    CPM_TRY(o->base.alloc(o->D));
    CPM_CUDA_TRY(cudaMemcpyAsync(o->base.p, t->base.p, o->D * 4, cudaMemcpyDeviceToDevice, stream()));
    CPM_TRY(o->w.alloc(12 * o->D));
    CPM_CUDA_TRY(cudaMemcpyAsync(o->w.p, t->w.p, 12 * o->D * 8, cudaMemcpyDeviceToDevice, stream()));
    CPM_TRY(o->flags.alloc(o->D));
    CPM_TRY(o->flags.zero());
    CPM_TRY(o->patch.alloc(o->D));
    CPM_CUDA_TRY(cudaMemsetAsync(o->patch.p, 0xff, o->D * 4, stream()));
    for (auto *b : {&o->p_eoff, &o->p_loff, &o->moved, &o->p_xcol, &o->lptr, &o->lcol}) CPM_TRY(b->alloc(1));
    CPM_TRY(o->p_emask.alloc(1));
    CPM_TRY(o->p_lmask.alloc(1));
    for (auto *b : {&o->p_xval, &o->lval, &o->ldiag}) CPM_TRY(b->alloc(1));
    for (auto *b : {&o->p_xval32, &o->lval32, &o->ldiag32}) CPM_TRY(b->alloc(1));
    o->h_identity.assign(o->D, 0);
    o->h_kind.assign(o->D, 0);
    o->h_ibc.assign(o->D, -1);
    CPM_TRY(t->cp.download(o->h_point, 3 * o->D));
    return 0;
}

__global__ void k_to_float(int64_t n, const double *__restrict__ a, float *__restrict__ b) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < n) b[i] = (float)a[i];
}

static int make_float_copies(cpm_opset_s *o) {
    auto conv = [&](DBuf<double> &a, DBuf<float> &b) -> int {
        CPM_TRY(b.alloc(a.n));
        k_to_float<<<(unsigned)((a.n + 255) / 256), 256, 0, stream()>>>((int64_t)a.n, a.p, b.p);
        CPM_CUDA_TRY(cudaGetLastError());
        return 0;
    };
    CPM_TRY(conv(o->w, o->w32));
    CPM_TRY(conv(o->w_ord, o->w_ord32));
    CPM_TRY(conv(o->p_xval, o->p_xval32));
    CPM_TRY(conv(o->lval, o->lval32));
    CPM_TRY(conv(o->ldiag, o->ldiag32));
    CPM_TRY(conv(o->pl_xval, o->pl_xval32));
    CPM_TRY(conv(o->pe_w, o->pe_w32));
    if (o->ov_w.n) CPM_TRY(conv(o->ov_w, o->ov_w32));
    return 0;
}

// Whole-tube Jcp normals (K7) on the plain (IBC-free) operator rows.
static int tube_normals(cpm_opset_s *base, std::vector<double> &normals) {
    cpm_tube_s *t = base->tube;
    const int64_t N = t->N;
    DBuf<double> g, J, nrm;
    CPM_TRY(g.alloc(9 * N));
    CPM_TRY(J.alloc(9 * N));
    CPM_TRY(nrm.alloc(3 * N));
    k_cp_gradients<<<(unsigned)((N + 255) / 256), 256, 0, stream()>>>(t->view(), N, t->key.p, t->cp.p, t->g.dx, g.p);
    k_extend9<<<(unsigned)((9 * N + 255) / 256), 256, 0, stream()>>>(base->view<double>(), g.p, J.p);
    k_jcp_normals<<<(unsigned)((N + 255) / 256), 256, 0, stream()>>>(N, J.p, nrm.p);
    CPM_CUDA_TRY(cudaGetLastError());
    CPM_TRY(nrm.download(normals, 3 * N));
    return 0;
}

int opset_tube_normals(cpm_opset_s *o) {
    std::vector<double> normals;
    CPM_TRY(tube_normals(o, normals));
    return o->normals.upload(normals);
}

static int build_ibc(cpm_opset_s *o, int n_ibc, const cpm_surface_desc *descs, const CpOverrides *ovr) {
    cpm_tube_s *t = o->tube;
    HostTube ht;
    CPM_TRY(ht.load(t));
    const int64_t N = ht.N;
    // the surface normals on the tube the IBC frames use: eigenvector 0 of the
    // symmetrised closest-point Jacobian, or x - cp (use_Jcp_surface_normals off)
    bool need_normals = false, need_xn = false;
    for (int c = 0; c < n_ibc; ++c)
        if (!descs[c].use_cp_diff_directions) (descs[c].use_Jcp_surface_normals ? need_normals : need_xn) = true;
    std::vector<double> normals, normals_x;
    if (need_normals) {
        CPM_TRY(tube_normals(o, normals));
        CPM_TRY(o->normals.upload(normals));
    }
    DBuf<double> dnx;
    if (need_xn) {
        normals_x = unoriented_normals(ht);
        CPM_TRY(dnx.upload(normals_x));
    }
    DBuf<double> xdev;
    CPM_TRY(xdev.alloc(3 * N));
    k_node_coords<<<(unsigned)((N + 255) / 256), 256, 0, stream()>>>(N, t->key.p, t->g.xstart, t->g.dx, xdev.p);
    CPM_CUDA_TRY(cudaGetLastError());
    std::vector<IBCData> ibs(n_ibc);
    for (int c = 0; c < n_ibc; ++c)
        CPM_TRY(build_ibc_data(t, ht, descs[c], descs[c].use_Jcp_surface_normals ? o->normals.p : dnx.p, xdev,
                               ovr ? &ovr->ibc[c] : nullptr, ovr ? &ovr->surface : nullptr, ibs[c]));
    o->ibc_desc.assign(descs, descs + n_ibc);
    o->ibc_verts.assign(n_ibc, {});
    o->ibc_prims.assign(n_ibc, {});
    for (int c = 0; c < n_ibc; ++c) {
        const cpm_surface_desc &d = descs[c];
        if (d.verts && d.nverts > 0) o->ibc_verts[c].assign(d.verts, d.verts + 3 * d.nverts);
        if (d.prims && d.nprims > 0) {
            const int64_t per = (d.kind == CPM_TRIANGULATION) ? 3 : 2;
            o->ibc_prims[c].assign(d.prims, d.prims + per * d.nprims);
        }
        o->ibc_desc[c].verts = o->ibc_verts[c].empty() ? nullptr : o->ibc_verts[c].data();
        o->ibc_desc[c].prims = o->ibc_prims[c].empty() ? nullptr : o->ibc_prims[c].data();
    }

    // column layout: IBCStartingColumns / TotalDOFs (src/IBCSubsets.cpp:74-116)
    o->n_ibc = n_ibc;
    o->col_start.assign(n_ibc, 0);
    o->dcol_start.assign(n_ibc, 0);
    if (n_ibc > 0) o->col_start[0] = o->dcol_start[0] = N;
    for (int c = 1; c < n_ibc; ++c) {
        // the reference numbers an order-1 IBC's Dirichlet value rows from
        // IdentityRowsStart too (IBCMatrixManipulations::DirichletValueRow), which is
        // past the last row once another IBC is 2nd order: mixed orders are refused
        if (ibs[c].order2 != ibs[0].order2)
            return fail(CPM_ERR_UNSUPPORTED, "IBCs of mixed boundary order are not implemented on the device path");
        o->col_start[c] = o->col_start[c - 1] + (int64_t)ibs[c - 1].dof_set.size();
        if (ibs[c].has_dir2) o->dcol_start[c] = o->dcol_start[c - 1] + ibs[c - 1].n_dir;
    }
    int64_t total = 0, num2 = 0, idstart = 0;
    for (int c = 0; c < n_ibc; ++c) {
        if (ibs[c].has_dir2) {
            idstart += 1;
            num2 += ibs[c].n_dir;
        }
        total += (int64_t)ibs[c].dof_set.size();
    }
    if (idstart) idstart = total;
    o->total_ibc = total;
    o->num2 = num2;
    o->identity_rows_start = idstart;
    const int64_t D = N + total + num2;
    o->D = D;
    auto value_row = [&](int c, int64_t i) -> int64_t {  // DirichletValueRow
        if (ibs[c].order2) return idstart + ibs[c].dir_sub[i] + o->dcol_start[c];
        return idstart + i + o->col_start[c];
    };

    // ---- host row structures
    std::vector<uint32_t> base(D, 0);
    std::vector<double> w(12 * D, 0.0);
    std::vector<uint8_t> flags(D, 0);
    std::vector<int32_t> patch(D, -1);
    std::vector<uint64_t> p_emask;
    std::vector<uint8_t> p_lmask;
    std::vector<int32_t> p_eoff, p_loff, moved, p_xcol, lptr{0}, lcol;
    std::vector<double> p_xval, lval, ldiag;
    {
        std::vector<uint32_t> tb;
        std::vector<double> tw;
        CPM_TRY(t->base.download(tb, N));
        CPM_TRY(t->w.download(tw, 12 * N));
        std::copy(tb.begin(), tb.end(), base.begin());
        std::copy(tw.begin(), tw.end(), w.begin());
    }
    std::vector<uint8_t> ident(D, 0);
    std::vector<int32_t> kind(D, 3), rowibc(D, -1), rowside(D, 0);
    std::vector<double> point(3 * D, 0.0);
    for (int64_t q = 0; q < N; ++q) {
        kind[q] = 0;
        for (int k = 0; k < 3; ++k) point[3 * q + k] = ht.cp[3 * q + k];
    }

    // ---- tube rows: moved E / L columns (MoveToIBCColumns, src/IBCMatrixManipulations.cpp:189-216),
    // on the device (k_tube_moves): masks and counts, then the targets at scanned offsets
    int64_t nmoved = 0;
    // every IBC's tagging on the device, for the TagStencils kernels
    std::vector<DBuf<int32_t>> d_tag_sub(n_ibc), d_dof_sub(n_ibc);
    std::vector<DBuf<uint8_t>> d_tag_bdy(n_ibc);
    std::vector<DBuf<double>> d_tag_dir(n_ibc);
    std::vector<IbcTagDev> hib(n_ibc);
    for (int c = 0; c < n_ibc; ++c) {
        const IBCData &ib = ibs[c];
        std::vector<int32_t> ts(ib.tag_sub.begin(), ib.tag_sub.end()), ds(ib.dof_sub.begin(), ib.dof_sub.end());
        CPM_TRY(d_tag_sub[c].upload(ts));
        CPM_TRY(d_dof_sub[c].upload(ds));
        std::vector<uint8_t> tb = ib.tag_bdy;
        std::vector<double> td = ib.tag_dir;
        if (tb.empty()) tb.push_back(0);
        if (td.empty()) td.assign(3, 0.0);
        CPM_TRY(d_tag_bdy[c].upload(tb));
        CPM_TRY(d_tag_dir[c].upload(td));
        hib[c] = IbcTagDev{d_tag_sub[c].p, d_tag_bdy[c].p, d_tag_dir[c].p, d_dof_sub[c].p, o->col_start[c]};
    }
    // extra targets (entries that move to several IBCs), per tube patch record
    std::vector<int32_t> ov_ptr{0}, ov_col, ov_s;
    std::vector<double> ov_w;
    if (n_ibc > 0) {
        DBuf<IbcTagDev> d_ibs;
        CPM_TRY(d_ibs.upload(hib));
        DBuf<uint64_t> d_em;
        DBuf<uint8_t> d_lm;
        DBuf<int32_t> d_cnt, d_xcnt, d_off, d_moved, d_xoff, d_xcol, d_xsd;
        CPM_TRY(d_em.alloc(N));
        CPM_TRY(d_lm.alloc(N));
        CPM_TRY(d_cnt.alloc(N));
        CPM_TRY(d_xcnt.alloc(2 * N));
        const unsigned nb = (unsigned)((N + 127) / 128);
        k_tube_moves<<<nb, 128, 0, stream()>>>(t->view(), N, t->key.p, t->base.p, d_ibs.p, n_ibc, d_em.p, d_lm.p, d_cnt.p,
                                               d_xcnt.p, nullptr, nullptr, nullptr, nullptr, nullptr);
        CPM_CUDA_TRY(cudaGetLastError());
        std::vector<uint64_t> em;
        std::vector<uint8_t> lm;
        std::vector<int32_t> cnt, xcnt;
        CPM_TRY(d_em.download(em, N));
        CPM_TRY(d_lm.download(lm, N));
        CPM_TRY(d_cnt.download(cnt, N));
        CPM_TRY(d_xcnt.download(xcnt, 2 * N));
        std::vector<int32_t> off(N), xoff(N);
        int64_t nx = 0;
        for (int64_t q = 0; q < N; ++q) {
            off[q] = (int32_t)nmoved;
            nmoved += cnt[q];
            xoff[q] = (int32_t)nx;
            nx += xcnt[2 * q] + xcnt[2 * q + 1];
            if (!em[q] && !lm[q]) continue;
            patch[q] = (int32_t)p_emask.size();
            p_emask.push_back(em[q]);
            p_lmask.push_back(lm[q]);
            p_eoff.push_back(off[q]);
            p_loff.push_back(off[q] + __builtin_popcountll(em[q]));
            p_xcol.push_back(0);
            p_xval.push_back(0.0);
            ov_ptr.push_back(ov_ptr.back() + xcnt[2 * q]);
            ov_ptr.push_back(ov_ptr.back() + xcnt[2 * q + 1]);
            if (em[q]) flags[q] |= F_EMOVE;
            if (lm[q]) flags[q] |= F_LMOVE;
            if (xcnt[2 * q] + xcnt[2 * q + 1]) flags[q] |= F_OVL;
        }
        if (nmoved > 0) {
            CPM_TRY(d_off.upload(off));
            CPM_TRY(d_moved.alloc(nmoved));
            int32_t *xc = nullptr, *xs = nullptr;
            if (nx > 0) {
                CPM_TRY(d_xoff.upload(xoff));
                CPM_TRY(d_xcol.alloc(nx));
                CPM_TRY(d_xsd.alloc(nx));
                xc = d_xcol.p;
                xs = d_xsd.p;
            }
            k_tube_moves<<<nb, 128, 0, stream()>>>(t->view(), N, t->key.p, t->base.p, d_ibs.p, n_ibc, nullptr, nullptr,
                                                   nullptr, nullptr, d_off.p, d_moved.p, d_xoff.p, xc, xs);
            CPM_CUDA_TRY(cudaGetLastError());
            CPM_TRY(d_moved.download(moved, nmoved));
            if (nx > 0) {
                CPM_TRY(d_xcol.download(ov_col, nx));
                CPM_TRY(d_xsd.download(ov_s, nx));
            }
        }
        // E extras carry the stencil weight of their point, as the patch entries do
        ov_w.assign(ov_col.size(), 0.0);
        for (int64_t q = 0; q < N; ++q) {
            if (patch[q] < 0) continue;
            const int pi = patch[q];
            for (int e = ov_ptr[2 * pi]; e < ov_ptr[2 * pi + 1]; ++e) {
                const int sx = ov_s[e], i = sx >> 4, j = (sx >> 2) & 3, k = sx & 3;
                ov_w[e] = (w[12 * q + i] * w[12 * q + 4 + j]) * w[12 * q + 8 + k];
            }
        }
    }
    const int64_t n_tube_patched = (int64_t)p_emask.size();

    // ---- IBC DOF rows and Dirichlet value rows
    const double Ldg = -6.0 / (ht.dx * ht.dx), Lof = 1.0 / (ht.dx * ht.dx);
    for (int c = 0; c < n_ibc; ++c) {
        const IBCData &ib = ibs[c];
        const int64_t nd = (int64_t)ib.dof_set.size();
        // the DOF rows' moved E entries and L columns, on the device (k_dof_moves)
        std::vector<uint64_t> dem;
        std::vector<int32_t> dcnt, dlc, dmoved;
        if (nd > 0) {
            std::vector<int32_t> dset(ib.dof_set.begin(), ib.dof_set.end());
            DBuf<int32_t> d_set, d_cnt, d_lc, d_off, d_mv;
            DBuf<uint32_t> d_base;
            DBuf<double> d_dir;
            DBuf<uint64_t> d_em;
            CPM_TRY(d_set.upload(dset));
            CPM_TRY(d_base.upload(ib.dof_rows.base));
            CPM_TRY(d_dir.upload(ib.dof_dir));
            CPM_TRY(d_em.alloc(nd));
            CPM_TRY(d_cnt.alloc(nd));
            CPM_TRY(d_lc.alloc(6 * nd));
            const unsigned nb = (unsigned)((nd + 127) / 128);
            k_dof_moves<<<nb, 128, 0, stream()>>>(t->view(), nd, t->key.p, d_set.p, d_base.p, d_dir.p, hib[c], d_em.p, d_cnt.p,
                                                  d_lc.p, nullptr, nullptr);
            CPM_CUDA_TRY(cudaGetLastError());
            CPM_TRY(d_em.download(dem, nd));
            CPM_TRY(d_cnt.download(dcnt, nd));
            CPM_TRY(d_lc.download(dlc, 6 * nd));
            std::vector<int32_t> doff(nd);
            int64_t tot = 0;
            for (int64_t i = 0; i < nd; ++i) {
                doff[i] = (int32_t)tot;
                tot += dcnt[i];
            }
            if (tot > 0) {
                CPM_TRY(d_off.upload(doff));
                CPM_TRY(d_mv.alloc(tot));
                k_dof_moves<<<nb, 128, 0, stream()>>>(t->view(), nd, t->key.p, d_set.p, d_base.p, d_dir.p, hib[c], nullptr,
                                                      nullptr, nullptr, d_off.p, d_mv.p);
                CPM_CUDA_TRY(cudaGetLastError());
                CPM_TRY(d_mv.download(dmoved, tot));
            }
            for (int64_t i = 0; i < nd; ++i) dcnt[i] = doff[i];  // now each DOF's first moved entry
        }
        for (int64_t i = 0; i < nd; ++i) {
            const int64_t row = o->col_start[c] + i;
            for (int k = 0; k < 3; ++k) point[3 * row + k] = ib.dof_cp[3 * i + k];
            rowibc[row] = c;
            rowside[row] = desc_side(ib, i);
            if (ib.dof_dirichlet(i) && !ib.order2) {
                // order-1 Dirichlet: identity DOF rows carrying the value.  Their L row
                // is still assembled (below): the reference's Lfull holds it, and only
                // identity_rows makes the solve skip it
                flags[row] = F_IDENT;
                ident[row] = 1;
                kind[row] = 2;
            } else {
            kind[row] = 1;
            // E row: E_ibc stencil (at cp-bar for order 2), tags with the DOF
            // direction and flip -1, scaled by -1 for Dirichlet
            // (AddExtensionIBCRows, src/IBCMatrixManipulations.cpp:118-186).
            base[row] = ib.dof_rows.base[i];
            for (int k = 0; k < 12; ++k) w[12 * row + k] = ib.dof_rows.w[12 * i + k];
            const uint64_t emask = dem[i];
            const int ne = __builtin_popcountll(emask);
            patch[row] = (int32_t)p_emask.size();
            p_emask.push_back(emask);
            p_lmask.push_back(0);
            p_eoff.push_back((int32_t)moved.size());
            moved.insert(moved.end(), dmoved.begin() + dcnt[i], dmoved.begin() + dcnt[i] + ne);
            p_loff.push_back((int32_t)moved.size());
            nmoved += ne;
            uint8_t f = F_LCSR;
            if (emask) f |= F_EMOVE;
            if (ib.dof_dirichlet(i)) {
                f |= F_ENEG | F_EXTRA;
                p_xcol.push_back((int32_t)value_row(c, i));
                p_xval.push_back(2.0);
            } else {
                p_xcol.push_back(0);
                p_xval.push_back(0.0);
            }
            flags[row] = f;
            }
            // L row (AddFiniteDifferenceIBCRows, src/IBCMatrixManipulations.cpp:219-251):
            // across the curve -> the original tube node; same side and in the DOF
            // subset -> that DOF's column; otherwise dropped.
            for (int d = 0; d < 6; ++d)
                if (dlc[6 * i + d] >= 0) {
                    lcol.push_back(dlc[6 * i + d]);
                    lval.push_back(Lof);
                }
            lptr.push_back((int32_t)lcol.size());
            ldiag.push_back(Ldg);
        }
    }
    // Dirichlet value rows of 2nd-order IBCs: identity
    for (int64_t row = N + total; row < D; ++row) {
        flags[row] = F_IDENT;
        lptr.push_back((int32_t)lcol.size());
        ldiag.push_back(0.0);
    }
    for (int c = 0; c < n_ibc; ++c)
        for (int64_t i = 0; i < (int64_t)ibs[c].dof_set.size(); ++i)
            if (ibs[c].dof_dirichlet(i)) {
                int64_t vr = value_row(c, i);
                ident[vr] = 1;
                kind[vr] = 2;
                rowibc[vr] = c;
                rowside[vr] = desc_side(ibs[c], i);
                for (int k = 0; k < 3; ++k) point[3 * vr + k] = ibs[c].dof_cp[3 * i + k];
            }
    if ((int64_t)lptr.size() != D - N + 1) return fail(CPM_ERR_CUDA, "internal: IBC row count mismatch");
    o->n_patched = n_tube_patched;
    o->n_moved = nmoved;

    // ---- upload
    CPM_TRY(o->base.upload(base));
    CPM_TRY(o->w.upload(w));
    CPM_TRY(o->flags.upload(flags));
    CPM_TRY(o->patch.upload(patch));
    if (p_emask.empty()) {
        p_emask.push_back(0);
        p_lmask.push_back(0);
        p_eoff.push_back(0);
        p_loff.push_back(0);
        p_xcol.push_back(0);
        p_xval.push_back(0);
    }
    if (moved.empty()) moved.push_back(0);
    if (lcol.empty()) {
        lcol.push_back(0);
        lval.push_back(0);
    }
    // the DOF rows' patch records (after the tube rows') have no extra targets
    ov_ptr.resize(2 * p_emask.size() + 1, ov_ptr.back());
    o->n_ov = (int64_t)ov_col.size();
    o->h_ov_ptr = ov_ptr;
    o->h_ov_col = ov_col;
    o->h_ov_s = ov_s;
    if (o->n_ov > 0) {
        CPM_TRY(o->ov_ptr.upload(ov_ptr));
        CPM_TRY(o->ov_col.upload(ov_col));
        CPM_TRY(o->ov_w.upload(ov_w));
    }
    CPM_TRY(o->p_emask.upload(p_emask));
    CPM_TRY(o->p_lmask.upload(p_lmask));
    CPM_TRY(o->p_eoff.upload(p_eoff));
    CPM_TRY(o->p_loff.upload(p_loff));
    CPM_TRY(o->moved.upload(moved));
    CPM_TRY(o->p_xcol.upload(p_xcol));
    CPM_TRY(o->p_xval.upload(p_xval));
    CPM_TRY(o->lptr.upload(lptr));
    CPM_TRY(o->lcol.upload(lcol));
    CPM_TRY(o->lval.upload(lval));
    CPM_TRY(o->ldiag.upload(ldiag));
    o->h_identity = ident;
    o->h_kind = kind;
    o->h_ibc = rowibc;
    o->h_side = rowside;
    o->h_point = point;
    o->tag_set.resize(n_ibc);
    o->dof_set.resize(n_ibc);
    o->dof_cp.resize(n_ibc);
    o->dof_cpdiff.resize(n_ibc);
    for (int c = 0; c < n_ibc; ++c) {
        o->tag_set[c] = ibs[c].tag_set;
        o->dof_set[c] = ibs[c].dof_set;
        o->dof_cp[c] = ibs[c].dof_cp;
        o->dof_cpdiff[c] = ibs[c].dof_cpdiff;
    }
    return 0;
}

// The six L columns of every tube row with IBC moves applied (-1: no neighbour).
__global__ void k_build_nbr6(OpView<double> op, int32_t *__restrict__ nbr6) {
    int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (r >= op.N) return;
    const uint32_t kk = op.key[r];
    const int i = unpack_i(kk), j = unpack_j(kk), k = unpack_k(kk);
    uint8_t lmask = 0;
    int loff = 0;
    if (op.flags[r] & F_LMOVE) {
        int pi = op.patch[r];
        lmask = op.p_lmask[pi];
        loff = op.p_loff[pi];
    }
    for (int d = 0; d < 6; ++d) {
        int col;
        if ((lmask >> d) & 1)
            col = op.moved[loff + __popc((unsigned)lmask & ((1u << d) - 1u))];
        else
            col = node_at(op.bv, i + (d == 0) - (d == 1), j + (d == 2) - (d == 3), k + (d == 4) - (d == 5));
        nbr6[6 * r + d] = col;
    }
}

// rows >= N: the IBC DOF rows' L columns (AddFiniteDifferenceIBCRows keeps at
// most the six neighbours, each with weight 1/dx^2 and the diagonal -6/dx^2),
// so every row's L has the tube-row form; identity rows get none.  err = 1 if a
// row has more than six off-diagonal entries.
__global__ void k_build_nbr6_ibc(OpView<double> op, int32_t *__restrict__ nbr6, int *__restrict__ err) {
    int64_t r = op.N + blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (r >= op.D) return;
    const int64_t q = r - op.N;
    const int e0 = op.lptr[q], e1 = op.lptr[q + 1];
    const bool ident = op.flags[r] & F_IDENT;
    if (!ident && e1 - e0 > 6) atomicOr(err, 1);
    for (int d = 0; d < 6; ++d) nbr6[6 * r + d] = (!ident && e0 + d < e1) ? op.lcol[e0 + d] : -1;
}

// 64 bulk stencil columns of each base group (s = 16 i + 4 j + k)
__global__ void k_group_cols(OpView<double> op, int64_t n_grp, int32_t *__restrict__ gcols) {
    int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (e >= 64 * n_grp) return;
    int64_t g = e >> 6;
    int s = (int)(e & 63);
    uint32_t b = op.base[op.ord[op.grp[g]]];
    int col = node_at(op.bv, unpack_i(b) + (s >> 4), unpack_j(b) + ((s >> 2) & 3), unpack_k(b) + (s & 3));
    gcols[e] = col >= 0 ? col : 0;  // missing stencil nodes are rejected at tube build time
}

// weights and flags in base-sorted row order
__global__ void k_sorted_rows(OpView<double> op, int64_t n_ord, double *__restrict__ w_ord, uint8_t *__restrict__ fl_ord) {
    int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (e >= 12 * n_ord) return;
    int64_t p = e / 12;
    int a = (int)(e % 12);
    int64_t r = op.ord[p];
    w_ord[e] = op.w[12 * r + a];
    if (a == 0) fl_ord[p] = op.flags[r];
}

// entries of the patch list: one thread per patched row, moved points in
// increasing stencil order s = 16 i + 4 j + k
__global__ void k_patch_entries(OpView<double> op, int64_t n_pl, int32_t *__restrict__ pe_new, int32_t *__restrict__ pe_old,
                                double *__restrict__ pe_w, int *__restrict__ err) {
    int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (q >= n_pl) return;
    const int r = op.pl_row[q];
    const int pi = op.patch[r];
    uint64_t em = (op.flags[r] & F_EMOVE) ? op.p_emask[pi] : 0ull;
    int mo = op.p_eoff[pi];
    const uint32_t b = op.base[r];
    const int bi = unpack_i(b), bj = unpack_j(b), bk = unpack_k(b);
    const double *w = op.w + 12 * (int64_t)r;
    int e = op.pl_off[q];
    while (em) {
        const int s = __ffsll((long long)em) - 1;
        em &= em - 1;
        const int i = s >> 4, j = (s >> 2) & 3, k = s & 3;
        const int old = node_at(op.bv, bi + i, bj + j, bk + k);
        if (old < 0) atomicOr(err, 1);
        pe_new[e] = op.moved[mo++];
        pe_old[e] = old < 0 ? 0 : old;
        pe_w[e] = (w[i] * w[4 + j]) * w[8 + k];
        ++e;
    }
}

// The patch list: rows whose E row is not the plain bulk stencil (moved
// columns, negation, an extra entry), so the 32-slot E passes can evaluate
// every row as bulk and correct these rows in a separate, parallel pass.
static int build_patch_list(cpm_opset_s *o, const std::vector<uint8_t> &flags) {
    const int64_t D = o->D;
    std::vector<int32_t> patch, p_xcol;
    std::vector<uint64_t> p_emask;
    std::vector<double> p_xval;
    std::vector<int32_t> rows, off{0}, xcol;
    std::vector<uint8_t> neg;
    std::vector<double> xval;
    if (o->patch.n >= (size_t)D) {
        CPM_TRY(o->patch.download(patch, D));
        CPM_TRY(o->p_emask.download(p_emask, o->p_emask.n));
        CPM_TRY(o->p_xcol.download(p_xcol, o->p_xcol.n));
        CPM_TRY(o->p_xval.download(p_xval, o->p_xval.n));
        for (int64_t r = 0; r < D; ++r) {
            const uint8_t f = flags[r];
            if ((f & F_IDENT) || !(f & (F_EMOVE | F_EXTRA | F_ENEG))) continue;
            const int pi = patch[r];
            if (pi < 0 || (size_t)pi >= p_emask.size()) return fail(CPM_ERR_CUDA, "internal: patched row without a patch record");
            rows.push_back((int32_t)r);
            off.push_back(off.back() + ((f & F_EMOVE) ? __builtin_popcountll(p_emask[pi]) : 0));
            const bool ex = (f & F_OVL) && o->h_ov_ptr[2 * pi + 1] > o->h_ov_ptr[2 * pi];
            neg.push_back((uint8_t)(((f & F_ENEG) ? 1 : 0) | (ex ? 2 : 0)));
            xcol.push_back((f & F_EXTRA) ? p_xcol[pi] : -1);
            xval.push_back((f & F_EXTRA) ? p_xval[pi] : 0.0);
        }
    }
    o->n_pl = (int64_t)rows.size();
    const int64_t ne = off.back();
    o->n_pe = ne;
    if (rows.empty()) {
        rows.push_back(0);
        neg.push_back(0);
        xcol.push_back(-1);
        xval.push_back(0.0);
    }
    CPM_TRY(o->pl_row.upload(rows));
    CPM_TRY(o->pl_off.upload(off));
    CPM_TRY(o->pl_neg.upload(neg));
    CPM_TRY(o->pl_xcol.upload(xcol));
    CPM_TRY(o->pl_xval.upload(xval));
    CPM_TRY(o->pe_new.alloc(std::max<int64_t>(1, ne)));
    CPM_TRY(o->pe_old.alloc(std::max<int64_t>(1, ne)));
    CPM_TRY(o->pe_w.alloc(std::max<int64_t>(1, ne)));
    if (o->n_pl > 0) {
        DBuf<int> err;
        CPM_TRY(err.alloc(1));
        CPM_TRY(err.zero());
        k_patch_entries<<<(unsigned)((o->n_pl + 255) / 256), 256, 0, stream()>>>(o->view<double>(), o->n_pl, o->pe_new.p,
                                                                                 o->pe_old.p, o->pe_w.p, err.p);
        CPM_CUDA_TRY(cudaGetLastError());
        std::vector<int> he;
        CPM_TRY(err.download(he, 1));
        if (he[0]) return fail(CPM_ERR_CUDA, "internal: a moved stencil point has no tube node");
    }
    return 0;
}

// Apply schedule: neighbour table, rows sorted by base point with their groups,
// identity rows.  Rows sharing a base point read the same 64 values of x.
static int build_schedule(cpm_opset_s *o) {
    const int64_t N = o->N, D = o->D;
    CPM_TRY(o->nbr6.alloc(6 * D));
    k_build_nbr6<<<(unsigned)((N + 255) / 256), 256, 0, stream()>>>(o->view<double>(), o->nbr6.p);
    CPM_CUDA_TRY(cudaGetLastError());
    if (D > N) {
        DBuf<int> err;
        CPM_TRY(err.alloc(1));
        CPM_TRY(err.zero());
        k_build_nbr6_ibc<<<(unsigned)((D - N + 255) / 256), 256, 0, stream()>>>(o->view<double>(), o->nbr6.p, err.p);
        CPM_CUDA_TRY(cudaGetLastError());
        std::vector<int> he;
        CPM_TRY(err.download(he, 1));
        if (he[0]) return fail(CPM_ERR_CUDA, "internal: an IBC L row has more than six off-diagonal entries");
    }
    std::vector<uint8_t> flags;
    std::vector<uint32_t> base;
    CPM_TRY(o->flags.download(flags, D));
    CPM_TRY(o->base.download(base, D));
    std::vector<std::pair<uint32_t, int32_t>> rows;
    std::vector<int32_t> ident;
    rows.reserve(D);
    for (int64_t r = 0; r < D; ++r) {
        if (flags[r] & F_IDENT)
            ident.push_back((int32_t)r);
        else
            rows.push_back({base[r], (int32_t)r});
    }
    std::sort(rows.begin(), rows.end());
    std::vector<int32_t> ord(rows.size()), grp;
    for (size_t p = 0; p < rows.size(); ++p) {
        ord[p] = rows[p].second;
        if (p == 0 || rows[p].first != rows[p - 1].first) grp.push_back((int32_t)p);
    }
    grp.push_back((int32_t)rows.size());
    o->n_ord = (int64_t)ord.size();
    o->n_grp = (int64_t)grp.size() - 1;
    o->n_ident = (int64_t)ident.size();
    if (ord.empty()) ord.push_back(0);
    if (ident.empty()) ident.push_back(0);
    CPM_TRY(o->ord.upload(ord));
    CPM_TRY(o->grp.upload(grp));
    CPM_TRY(o->ident.upload(ident));
    // per group: its 64 bulk stencil columns; per sorted row: weights and flags
    CPM_TRY(o->gcols.alloc(64 * std::max<int64_t>(1, o->n_grp)));
    CPM_TRY(o->w_ord.alloc(12 * std::max<int64_t>(1, o->n_ord)));
    CPM_TRY(o->fl_ord.alloc(std::max<int64_t>(1, o->n_ord)));
    if (o->n_grp > 0) {
        k_group_cols<<<(unsigned)((64 * o->n_grp + 255) / 256), 256, 0, stream()>>>(o->view<double>(), o->n_grp, o->gcols.p);
        k_sorted_rows<<<(unsigned)((12 * o->n_ord + 255) / 256), 256, 0, stream()>>>(o->view<double>(), o->n_ord, o->w_ord.p,
                                                                                    o->fl_ord.p);
        CPM_CUDA_TRY(cudaGetLastError());
    }
    return build_patch_list(o, flags);
}

}  // namespace cpm

using namespace cpm;

static int opset_create(cpm_tube_t t, int32_t n_ibc, const cpm_surface_desc *ibcs, const CpOverrides *ovr, cpm_opset_t *out) {
    if (!t || !out || n_ibc < 0 || (n_ibc > 0 && !ibcs)) return fail(CPM_ERR_INVALID_ARG, "invalid arguments");
    *out = nullptr;
    cpm_opset_s *o = new cpm_opset_s();
    o->tube = t;
    int rc = build_base(o);
    if (!rc && n_ibc > 0) rc = build_ibc(o, n_ibc, ibcs, ovr);
    if (!rc) rc = build_schedule(o);
    if (!rc) rc = make_float_copies(o);
    if (!rc) {
        cudaError_t e = cudaStreamSynchronize(stream());
        if (e != cudaSuccess) rc = fail(CPM_ERR_CUDA, cudaGetErrorString(e));
    }
    if (rc) {
        delete o;
        return rc;
    }
    *out = o;
    return 0;
}

extern "C" int cpm_opset_create(cpm_tube_t t, int32_t n_ibc, const cpm_surface_desc *ibcs, cpm_opset_t *out) {
    return opset_create(t, n_ibc, ibcs, nullptr, out);
}

extern "C" int cpm_opset_create_from_cp(cpm_tube_t t, int32_t n_ibc, const cpm_surface_desc *ibcs,
                                        const cpm_cp_table *ibc_cp, const cpm_cp_table *surface_cp, cpm_opset_t *out) {
    CpOverrides ovr;
    ovr.ibc.resize(n_ibc > 0 ? n_ibc : 0);
    for (int c = 0; c < n_ibc && ibc_cp; ++c) ovr.ibc[c].load(&ibc_cp[c]);
    ovr.surface.load(surface_cp);
    CPM_TRY(opset_create(t, n_ibc, ibcs, &ovr, out));
    (*out)->cp_ovr = std::make_shared<CpOverrides>(std::move(ovr));
    return 0;
}

// the operator of the nearest-node baselines (PoissonWithIBCNearest::Initialize,
// problems/PoissonWithIBCNearest.cpp:73-89): plain L and E of the tube (no IBC
// columns) with identity rows at the given tube rows (device indices), which
// hold Dirichlet values
namespace cpm {
static int build_point_batch(cpm_opset_s *o, int n_src, const double *sources, PointBatchInfo &info) {
    cpm_tube_s *t = o->tube;
    HostTube ht;
    CPM_TRY(ht.load(t));
    const int64_t N = ht.N;
    std::vector<double> normals;
    CPM_TRY(tube_normals(o, normals));
    CPM_TRY(o->normals.upload(normals));
    DBuf<double> xdev;
    CPM_TRY(xdev.alloc(3 * N));
    k_node_coords<<<(unsigned)((N + 255) / 256), 256, 0, stream()>>>(N, t->key.p, t->g.xstart, t->g.dx, xdev.p);
    CPM_CUDA_TRY(cudaGetLastError());
    std::vector<uint32_t> base;
    std::vector<double> w;
    CPM_TRY(t->base.download(base, N));
    CPM_TRY(t->w.download(w, 12 * N));
    // per tube row: its records {slot, kind, replaced column, DOF column} and E weights
    std::vector<std::vector<std::pair<int4, double>>> recs(N);
    int64_t M = 0;
    info.dof_set.assign(n_src, {});
    info.dof_cpdiff.assign(n_src, {});
    for (int k = 0; k < n_src; ++k) {
        // GeodesicDistance's point IBC (cpm_geodesic_create): order 1, Dirichlet, on_ibc_tolerance 0.1 dx^2
        cpm_surface_desc pd;
        memset(&pd, 0, sizeof(pd));
        pd.kind = CPM_POINT;
        pd.nparams = 3;
        for (int d = 0; d < 3; ++d) pd.params[d] = sources[3 * k + d];
        pd.bbox[0] = t->surf.desc.bbox[0];
        pd.bbox[1] = t->surf.desc.bbox[1];
        pd.boundary_order = 1;
        pd.use_Jcp_surface_normals = 1;
        pd.on_ibc_tolerance = 0.1 * t->g.dx * t->g.dx;
        pd.dof_radius_scale = 1.0;
        IBCData ib;
        CPM_TRY(build_ibc_data(t, ht, pd, o->normals.p, xdev, nullptr, nullptr, ib));
        M = std::max<int64_t>(M, (int64_t)ib.dof_set.size());
        // MoveToIBCColumns for this slot's IBC alone (one IBC: a stencil entry moves at most once)
        for (size_t i = 0; i < ib.tag_set.size(); ++i) {
            const int64_t q = ib.tag_set[i];
            const double *dir = &ib.tag_dir[3 * i];
            for (int sidx = 0; sidx < 64; ++sidx) {
                const int a = sidx >> 4, b = (sidx >> 2) & 3, c = sidx & 3;
                const int col = ht.node(unpack_i(base[q]) + a, unpack_j(base[q]) + b, unpack_k(base[q]) + c);
                if (col >= 0 && tagged(ib, dir, col, 1.0) && ib.dof_sub[col] >= 0)
                    recs[q].push_back({make_int4(k, 0, col, (int)(N + ib.dof_sub[col])),
                                       (w[12 * q + a] * w[12 * q + 4 + b]) * w[12 * q + 8 + c]});
            }
            for (int d = 0; d < 6; ++d) {
                const int col = ht.nbr(q, d);
                if (col >= 0 && tagged(ib, dir, col, 1.0) && ib.dof_sub[col] >= 0)
                    recs[q].push_back({make_int4(k, 1, col, (int)(N + ib.dof_sub[col])), 0.0});
            }
        }
        info.dof_set[k] = ib.dof_set;
        info.dof_cpdiff[k] = ib.dof_cpdiff;
    }
    // rows N .. N + M: identity rows (slot k's DOF values)
    const int64_t D = N + M;
    o->D = D;
    std::vector<uint8_t> flags(D, 0), ident(D, 0);
    for (int64_t r = N; r < D; ++r) {
        flags[r] = F_IDENT;
        ident[r] = 1;
    }
    std::vector<int32_t> sp_ptr(D + 1, 0), sp_rows;
    std::vector<int4> sp_rec;
    std::vector<double> sp_w;
    for (int64_t q = 0; q < D; ++q) {
        sp_ptr[q] = (int32_t)sp_rec.size();
        if (q < N && !recs[q].empty()) {
            flags[q] |= F_SLOTP;
            sp_rows.push_back((int32_t)q);
            for (auto &e : recs[q]) {
                sp_rec.push_back(e.first);
                sp_w.push_back(e.second);
            }
        }
    }
    sp_ptr[D] = (int32_t)sp_rec.size();
    o->n_sp_rows = (int64_t)sp_rows.size();
    if (sp_rows.empty()) sp_rows.push_back(0);
    if (sp_rec.empty()) {
        sp_rec.push_back(make_int4(-1, 0, 0, 0));
        sp_w.push_back(0.0);
    }
    std::vector<uint32_t> base_d(D, 0);
    std::vector<double> w_d(12 * D, 0.0);
    std::copy(base.begin(), base.end(), base_d.begin());
    std::copy(w.begin(), w.end(), w_d.begin());
    std::vector<int32_t> patch(D, -1), lptr(D - N + 1, 0);
    std::vector<double> ldiag(D - N + 1, 0.0);
    CPM_TRY(o->base.upload(base_d));
    CPM_TRY(o->w.upload(w_d));
    CPM_TRY(o->flags.upload(flags));
    CPM_TRY(o->patch.upload(patch));
    CPM_TRY(o->lptr.upload(lptr));
    CPM_TRY(o->ldiag.upload(ldiag));
    CPM_TRY(o->sp_ptr.upload(sp_ptr));
    CPM_TRY(o->sp_rows.upload(sp_rows));
    CPM_TRY(o->sp_rec.upload(sp_rec));
    CPM_TRY(o->sp_w.upload(sp_w));
    std::vector<float> sp_w32(sp_w.begin(), sp_w.end());
    CPM_TRY(o->sp_w32.upload(sp_w32));
    o->h_identity = ident;
    o->h_kind.assign(D, 0);
    o->h_ibc.assign(D, -1);
    for (int64_t r = N; r < D; ++r) o->h_kind[r] = 2;
    o->h_point.resize(3 * D, 0.0);
    return 0;
}

int opset_create_point_batch(cpm_tube_s *t, int n_src, const double *sources, cpm_opset_s **out, PointBatchInfo &info) {
    if (!t || !out || n_src < 1 || n_src > 32 || !sources) return fail(CPM_ERR_INVALID_ARG, "point batch: 1 to 32 sources");
    *out = nullptr;
    cpm_opset_s *o = new cpm_opset_s();
    o->tube = t;
    int rc = build_base(o);
    if (!rc) rc = build_point_batch(o, n_src, sources, info);
    if (!rc) rc = build_schedule(o);
    if (!rc) rc = make_float_copies(o);
    if (!rc) {
        cudaError_t e = cudaStreamSynchronize(stream());
        if (e != cudaSuccess) rc = fail(CPM_ERR_CUDA, cudaGetErrorString(e));
    }
    if (rc) {
        delete o;
        return rc;
    }
    *out = o;
    return 0;
}
}  // namespace cpm

extern "C" int cpm_opset_create_identity(cpm_tube_t t, int64_t n_rows, const int64_t *rows, cpm_opset_t *out) {
    if (!t || !out || n_rows < 0 || (n_rows > 0 && !rows)) return fail(CPM_ERR_INVALID_ARG, "invalid arguments");
    *out = nullptr;
    cpm_opset_s *o = new cpm_opset_s();
    o->tube = t;
    int rc = build_base(o);
    if (!rc) {
        std::vector<uint8_t> fl(o->D, 0);
        for (int64_t i = 0; i < n_rows && !rc; ++i) {
            if (rows[i] < 0 || rows[i] >= o->D) {
                rc = fail(CPM_ERR_INVALID_ARG, "identity row outside the tube");
                break;
            }
            fl[rows[i]] = F_IDENT;
            o->h_identity[rows[i]] = 1;
            o->h_kind[rows[i]] = 2;
        }
        if (!rc) rc = o->flags.upload(fl);
    }
    if (!rc) rc = build_schedule(o);
    if (!rc) rc = make_float_copies(o);
    if (!rc) {
        cudaError_t e = cudaStreamSynchronize(stream());
        if (e != cudaSuccess) rc = fail(CPM_ERR_CUDA, cudaGetErrorString(e));
    }
    if (rc) {
        delete o;
        return rc;
    }
    *out = o;
    return 0;
}

extern "C" int cpm_opset_sizes(cpm_opset_t o, int64_t *s) {
    if (!o || !s) return fail(CPM_ERR_INVALID_ARG, "null argument");
    s[0] = o->D;
    s[1] = o->N;
    s[2] = o->total_ibc;
    s[3] = o->num2;
    s[4] = o->n_ibc;
    s[5] = o->n_patched;
    s[6] = o->n_moved;
    s[7] = o->n_pl;
    s[8] = o->n_pe;
    return 0;
}

extern "C" int cpm_opset_rows(cpm_opset_t o, uint8_t *identity, int32_t *kind, int32_t *ibc, double *point) {
    if (!o) return fail(CPM_ERR_INVALID_ARG, "null opset");
    for (int64_t r = 0; r < o->D; ++r) {
        if (identity) identity[r] = o->h_identity[r];
        if (kind) kind[r] = o->h_kind[r];
        if (ibc) ibc[r] = o->h_ibc[r];
        if (point)
            for (int k = 0; k < 3; ++k) point[3 * r + k] = o->h_point[3 * r + k];
    }
    return 0;
}

extern "C" int cpm_opset_row_sides(cpm_opset_t o, int32_t *side) {
    if (!o || !side) return fail(CPM_ERR_INVALID_ARG, "null argument");
    for (int64_t r = 0; r < o->D; ++r) side[r] = (r < (int64_t)o->h_side.size()) ? o->h_side[r] : 0;
    return 0;
}

extern "C" int cpm_opset_ibc_sizes(cpm_opset_t o, int32_t c, int64_t *s) {
    if (!o || c < 0 || c >= o->n_ibc || !s) return fail(CPM_ERR_INVALID_ARG, "invalid IBC index");
    s[0] = (int64_t)o->tag_set[c].size();
    s[1] = (int64_t)o->dof_set[c].size();
    s[2] = o->col_start[c];
    s[3] = o->dcol_start[c];
    s[4] = o->identity_rows_start;
    return 0;
}

extern "C" int cpm_opset_ibc_export(cpm_opset_t o, int32_t c, int64_t *tag_set, int64_t *dof_set, double *dof_cp) {
    if (!o || c < 0 || c >= o->n_ibc) return fail(CPM_ERR_INVALID_ARG, "invalid IBC index");
    if (tag_set) std::copy(o->tag_set[c].begin(), o->tag_set[c].end(), tag_set);
    if (dof_set) std::copy(o->dof_set[c].begin(), o->dof_set[c].end(), dof_set);
    if (dof_cp) std::copy(o->dof_cp[c].begin(), o->dof_cp[c].end(), dof_cp);
    return 0;
}

// Lfull / Efull as CSR (sorted columns) reconstructed from the device rows.
extern "C" int cpm_opset_export_csr(cpm_opset_t o, int32_t which, int64_t *nnz, int64_t *ptr, int64_t *idx, double *val) {
    if (!o || !nnz || !(which == 0 || which == 1 || (which >= 5 && which <= 7))) return fail(CPM_ERR_INVALID_ARG, "invalid arguments");
    HostTube ht;
    CPM_TRY(ht.load(o->tube));
    const int64_t D = o->D, N = o->N;
    std::vector<uint32_t> base;
    std::vector<double> w, p_xval, lval, ldiag;
    std::vector<uint8_t> flags, p_lmask;
    std::vector<int32_t> patch, p_eoff, p_loff, moved, p_xcol, lptr, lcol;
    std::vector<uint64_t> p_emask;
    CPM_TRY(o->base.download(base, D));
    CPM_TRY(o->w.download(w, 12 * D));
    CPM_TRY(o->flags.download(flags, D));
    CPM_TRY(o->patch.download(patch, D));
    CPM_TRY(o->p_emask.download(p_emask, o->p_emask.n));
    CPM_TRY(o->p_lmask.download(p_lmask, o->p_lmask.n));
    CPM_TRY(o->p_eoff.download(p_eoff, o->p_eoff.n));
    CPM_TRY(o->p_loff.download(p_loff, o->p_loff.n));
    CPM_TRY(o->moved.download(moved, o->moved.n));
    CPM_TRY(o->p_xcol.download(p_xcol, o->p_xcol.n));
    CPM_TRY(o->p_xval.download(p_xval, o->p_xval.n));
    CPM_TRY(o->lptr.download(lptr, o->lptr.n));
    CPM_TRY(o->lcol.download(lcol, o->lcol.n));
    CPM_TRY(o->lval.download(lval, o->lval.n));
    CPM_TRY(o->ldiag.download(ldiag, o->ldiag.n));
    const double Ldg = -6.0 / (o->dx * o->dx), Lof = 1.0 / (o->dx * o->dx);
    std::vector<std::pair<int64_t, double>> row;
    int64_t count = 0;
    if (ptr) ptr[0] = 0;
    for (int64_t r = 0; r < D; ++r) {
        row.clear();
        uint8_t f = flags[r];
        // identity rows are identity rows of Efull (Helpers::SetIdentityRows on E, src/Helpers.cpp:403-431);
        // Lfull keeps the L rows of the tube and of the IBC DOFs, and the 2nd-order Dirichlet value rows
        // hold their 1 (src/IBCMatrixManipulations.cpp:54-62)
        const bool ident_row = (f & F_IDENT) && (which == 1 || r >= N + o->total_ibc);
        if (which >= 5) {
            // the gradient matrix Dc_d of the tube rows (FDMatrices::BuildGradientMatrices,
            // src/FDMatrices.cpp:66-92): (-1)^nbr 0.5 at the +/- e_d neighbours, then / dx
            if (r < N)
                for (int e = 0; e < 2; ++e) {
                    const int col = ht.nbr(r, 2 * (which - 5) + e);
                    if (col >= 0) row.push_back({col, (e ? -0.5 : 0.5) / o->dx});
                }
        } else if (ident_row) {
            row.push_back({r, 1.0});
        } else if (which == 1) {
            int pi = patch[r];
            uint64_t emask = (pi >= 0) ? p_emask[pi] : 0;
            int eoff = (pi >= 0) ? p_eoff[pi] : 0;
            uint32_t b = base[r];
            double sg = (f & F_ENEG) ? -1.0 : 1.0;
            for (int s = 0; s < 64; ++s) {
                int i = s >> 4, j = (s >> 2) & 3, k = s & 3;
                int64_t col = ((emask >> s) & 1ull) ? moved[eoff + __builtin_popcountll(emask & ((1ull << s) - 1ull))]
                                                    : ht.node(unpack_i(b) + i, unpack_j(b) + j, unpack_k(b) + k);
                row.push_back({col, sg * (w[12 * r + 8 + k] * w[12 * r + 4 + j] * w[12 * r + i])});
            }
            if (f & F_OVL)  // the further copies of entries that move to several IBCs
                for (int e = o->h_ov_ptr[2 * pi]; e < o->h_ov_ptr[2 * pi + 1]; ++e) {
                    const int sx = o->h_ov_s[e], i = sx >> 4, j = (sx >> 2) & 3, k = sx & 3;
                    row.push_back({o->h_ov_col[e], sg * (w[12 * r + 8 + k] * w[12 * r + 4 + j] * w[12 * r + i])});
                }
            if (f & F_EXTRA) row.push_back({p_xcol[pi], p_xval[pi]});
        } else if (r < N) {
            int pi = patch[r];
            uint8_t lm = (pi >= 0) ? p_lmask[pi] : 0;
            int loff = (pi >= 0) ? p_loff[pi] : 0;
            row.push_back({r, Ldg});
            for (int d = 0; d < 6; ++d) {
                int64_t col = ((lm >> d) & 1) ? moved[loff + __builtin_popcount((unsigned)lm & ((1u << d) - 1u))] : ht.nbr(r, d);
                if (col >= 0) row.push_back({col, Lof});
            }
            if (f & F_OVL)
                for (int e = o->h_ov_ptr[2 * pi + 1]; e < o->h_ov_ptr[2 * pi + 2]; ++e) row.push_back({o->h_ov_col[e], Lof});
        } else {
            int64_t q = r - N;
            row.push_back({r, ldiag[q]});
            for (int e = lptr[q]; e < lptr[q + 1]; ++e) row.push_back({lcol[e], lval[e]});
        }
        std::sort(row.begin(), row.end(),
                  [](const std::pair<int64_t, double> &a, const std::pair<int64_t, double> &b) { return a.first < b.first; });
        if (idx)
            for (size_t e = 0; e < row.size(); ++e) {
                idx[count + e] = row[e].first;
                val[count + e] = row[e].second;
            }
        count += (int64_t)row.size();
        if (ptr) ptr[r + 1] = count;
    }
    *nnz = count;
    return 0;
}

extern "C" int cpm_opset_destroy(cpm_opset_t o) {
    delete o;
    return 0;
}

// GetPlotInterpMatrix + AddIBCPlotInterpolation (src/Helpers.cpp:97-103;
// src/IBCMatrixManipulations.cpp:84-106 with PlotPointsCPDiff :254-416, the
// non-oriented branch): each evaluation point's 64 interpolation entries, with
// the stencil nodes that lie across an IBC from the point moved to that IBC's
// DOF columns, as the operator's E rows are.  The IBC subsets are derived again
// from the stored descriptions (this is a post-processing query, not a solve).
// the evaluation rows: per point its 64 (column, value) entries with the moves
// applied, and the further copies of entries that lie across several IBCs as
// (point, column, value) extras in point and stencil order
struct PlotExtras {
    std::vector<int64_t> row, col;
    std::vector<double> val;
};

static int plot_interp_rows(cpm_opset_t op, int64_t n, const double *xp, int64_t *cols, double *vals, PlotExtras &ex) {
    CPM_TRY(cpm_interp_query(op->tube, n, xp, cols, vals));
    for (int64_t e = 0; e < 64 * n; ++e)
        if (cols[e] < 0) return fail(CPM_ERR_BASEPOINT_OUTSIDE_TUBE, "plot interpolation stencil leaves the tube");
    const int n_ibc = (int)op->n_ibc;
    if (n_ibc == 0) return 0;
    cpm_tube_s *t = op->tube;
    HostTube ht;
    CPM_TRY(ht.load(t));
    const int64_t N = ht.N;
    const double r = ht.radius;
    std::vector<double> normals, normals_x;
    bool need_normals = false, need_xn = false;
    for (int c = 0; c < n_ibc; ++c)
        if (!op->ibc_desc[c].use_cp_diff_directions) (op->ibc_desc[c].use_Jcp_surface_normals ? need_normals : need_xn) = true;
    DBuf<double> dn, dnx;
    const double *normals_dev = op->normals.p;
    if (need_normals) {
        if (op->normals.n >= (size_t)(3 * N)) {
            CPM_TRY(op->normals.download(normals, 3 * N));
        } else {
            CPM_TRY(tube_normals(op, normals));
            CPM_TRY(dn.upload(normals));
            normals_dev = dn.p;
        }
    }
    if (need_xn) {
        normals_x = unoriented_normals(ht);
        CPM_TRY(dnx.upload(normals_x));
    }
    DBuf<double> xdev;
    CPM_TRY(xdev.alloc(3 * N));
    k_node_coords<<<(unsigned)((N + 255) / 256), 256, 0, stream()>>>(N, t->key.p, t->g.xstart, t->g.dx, xdev.p);
    CPM_CUDA_TRY(cudaGetLastError());
    std::vector<IBCData> ibs(n_ibc);
    const CpOverrides *ovr = op->cp_ovr.get();
    for (int c = 0; c < n_ibc; ++c)
        CPM_TRY(build_ibc_data(t, ht, op->ibc_desc[c], op->ibc_desc[c].use_Jcp_surface_normals ? normals_dev : dnx.p, xdev,
                               ovr ? &ovr->ibc[c] : nullptr, ovr ? &ovr->surface : nullptr, ibs[c]));
    std::vector<double> hx(xp, xp + 3 * n);
    DBuf<double> dxp;
    CPM_TRY(dxp.upload(hx));
    // per IBC: the points within 2r of it and their tagging directions
    std::vector<std::vector<int64_t>> sub(n_ibc, std::vector<int64_t>(n, -1));
    std::vector<std::vector<double>> dirs(n_ibc);
    for (int c = 0; c < n_ibc; ++c) {
        const cpm_surface_desc &desc = op->ibc_desc[c];
        SurfaceObj s;
        CPM_TRY(surface_init(s, &desc, r));
        DBuf<double> dcp, dd;
        CPM_TRY(dcp.alloc(3 * n));
        CPM_TRY(dd.alloc(n));
        CPM_TRY(closest_points_dev(s.params(), n, dxp.p, dcp.p, dd.p, 2.0 * r * (1.0 + 1e-12)));
        std::vector<double> cpc, dist;
        CPM_TRY(dcp.download(cpc, 3 * n));
        CPM_TRY(dd.download(dist, n));
        std::vector<double> scp, sdiff;
        int64_t count = 0;
        for (int64_t i = 0; i < n; ++i) {
            double cd[3];
            for (int k = 0; k < 3; ++k) cd[k] = hx[3 * i + k] - cpc[3 * i + k];
            if (!(std::sqrt(hdot(cd, cd)) < 2.0 * r)) continue;
            sub[c][i] = count++;
            for (int k = 0; k < 3; ++k) {
                scp.push_back(cpc[3 * i + k]);
                sdiff.push_back(cd[k]);
            }
        }
        for (int64_t i = 0; i < n; ++i) {
            const int64_t si = sub[c][i];
            if (si < 0 || !(std::sqrt(hdot(&sdiff[3 * si], &sdiff[3 * si])) < desc.on_ibc_tolerance)) continue;
            const int64_t nearest = ht.nearest(&hx[3 * i]);
            if (nearest >= 0 && ibs[c].tag_sub[nearest] >= 0)
                for (int k = 0; k < 3; ++k) sdiff[3 * si + k] = ibs[c].tag_cpdiff[3 * ibs[c].tag_sub[nearest] + k];
        }
        QueryRows qs;
        CPM_TRY(query_weights(t, scp, qs));
        const std::vector<double> bn = interp_unoriented(ht, qs, ibs[c].tag_binormal, &ibs[c].tag_sub);
        dirs[c].assign(3 * count, 0.0);
        for (int64_t si = 0; si < count; ++si) {
            const double b = hdot(&bn[3 * si], &sdiff[3 * si]);
            for (int k = 0; k < 3; ++k) dirs[c][3 * si + k] = b * bn[3 * si + k];
        }
    }
    // TagStencils + MoveToIBCColumns on the evaluation rows
    for (int64_t i = 0; i < n; ++i)
        for (int e = 0; e < 64; ++e) {
            const int col = (int)cols[64 * i + e];
            int hits = 0;
            for (int c = 0; c < n_ibc; ++c) {
                const int64_t si = sub[c][i];
                if (si < 0) continue;
                if (tagged(ibs[c], &dirs[c][3 * si], col, 1.0) && ibs[c].dof_sub[col] >= 0) {
                    const int64_t tgt = op->col_start[c] + ibs[c].dof_sub[col];
                    if (hits++ == 0) {
                        cols[64 * i + e] = tgt;
                    } else {  // MoveToIBCColumns: one copy of the entry per IBC
                        ex.row.push_back(i);
                        ex.col.push_back(tgt);
                        ex.val.push_back(vals[64 * i + e]);
                    }
                }
            }
        }
    return 0;
}

extern "C" int cpm_opset_plot_interp(cpm_opset_t op, int64_t n, const double *xp, int64_t *cols, double *vals) {
    if (!op || n < 0 || (n > 0 && (!xp || !cols || !vals))) return fail(CPM_ERR_INVALID_ARG, "invalid arguments");
    if (n == 0) return 0;
    PlotExtras ex;
    CPM_TRY(plot_interp_rows(op, n, xp, cols, vals, ex));
    if (!ex.row.empty())
        return fail(CPM_ERR_UNSUPPORTED, "an evaluation stencil entry lies across two IBCs: use cpm_opset_plot_interp_csr");
    return 0;
}

// the same rows as CSR: each point's 64 entries, then its extra copies
extern "C" int cpm_opset_plot_interp_csr(cpm_opset_t op, int64_t n, const double *xp, int64_t *nnz, int64_t *ptr,
                                         int64_t *cols, double *vals) {
    if (!op || n < 0 || !nnz || (n > 0 && !xp)) return fail(CPM_ERR_INVALID_ARG, "invalid arguments");
    std::vector<int64_t> c64(64 * (size_t)n);
    std::vector<double> v64(64 * (size_t)n);
    PlotExtras ex;
    if (n > 0) CPM_TRY(plot_interp_rows(op, n, xp, c64.data(), v64.data(), ex));
    *nnz = 64 * n + (int64_t)ex.row.size();
    if (!ptr) return 0;
    if (*nnz > 0 && (!cols || !vals)) return fail(CPM_ERR_INVALID_ARG, "invalid arguments");
    size_t x = 0;
    int64_t k = 0;
    ptr[0] = 0;
    for (int64_t i = 0; i < n; ++i) {
        for (int e = 0; e < 64; ++e, ++k) {
            cols[k] = c64[64 * i + e];
            vals[k] = v64[64 * i + e];
        }
        for (; x < ex.row.size() && ex.row[x] == i; ++x, ++k) {
            cols[k] = ex.col[x];
            vals[k] = ex.val[x];
        }
        ptr[i + 1] = k;
    }
    return 0;
}

// Surface::xp() of an IBC curve (Surface::GetSurfaceParameterization,
// src/Surface.cpp:194-216): a Circle3D's 100 parameter points, a Point, or a
// polyline's vertices.  n in, the count out; xp NULL queries the count.
extern "C" int cpm_ibc_plot_points(const cpm_surface_desc *ibc, int64_t *n, double *xp) {
    if (!ibc || !n) return fail(CPM_ERR_INVALID_ARG, "invalid arguments");
    int64_t cnt = 0;
    if (ibc->kind == CPM_CIRCLE3D)
        cnt = CIRCLE_NP;
    else if (ibc->kind == CPM_POINT)
        cnt = 1;
    else if (ibc->kind == CPM_POLYLINE || ibc->kind == CPM_TRIANGULATION)
        cnt = ibc->nverts;
    else
        return fail(CPM_ERR_UNSUPPORTED, "plot points of this IBC kind are not offered");
    if (!xp) {
        *n = cnt;
        return 0;
    }
    if (*n < cnt) return fail(CPM_ERR_INVALID_ARG, "xp holds fewer points than the curve has");
    for (int64_t i = 0; i < cnt; ++i) {
        if (ibc->kind == CPM_CIRCLE3D)
            circle_point(ibc->params, i, xp + 3 * i);
        else if (ibc->kind == CPM_POINT)
            for (int k = 0; k < 3; ++k) xp[3 * i + k] = ibc->params[k];
        else
            for (int k = 0; k < 3; ++k) xp[3 * i + k] = ibc->verts[3 * i + k];
    }
    *n = cnt;
    return 0;
}

// Tube::NearestTubeIndex (src/Tube.h:116-121): the tube node at the grid point
// nearest each x (device index), or -1 where that grid point is not in the tube
extern "C" int cpm_tube_nearest(cpm_tube_t t, int64_t n, const double *x, int64_t *idx) {
    if (!t || n < 0 || (n > 0 && (!x || !idx))) return fail(CPM_ERR_INVALID_ARG, "invalid arguments");
    if (n == 0) return 0;
    HostTube ht;
    CPM_TRY(ht.load(t));
    for (int64_t i = 0; i < n; ++i) idx[i] = ht.nearest(x + 3 * i);
    return 0;
}
