// ORACLE — test infrastructure only. Not part of the product library.
#include "ibc.h"

#include <cmath>
#include <limits>
#include <stdexcept>

namespace cpmref {

// ---------------------------------------------------------------------------
// Cyclic Jacobi eigen-solver for a symmetric 3x3 matrix (Golub & Van Loan 8.5.2,
// with the rotation of Rutishauser's stable formulation).  Sorted ascending.
Eig3 SymmetricEigen3(const double Ain[3][3]) {
    double a[3][3], v[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) a[i][j] = Ain[i][j];
    for (int sweep = 0; sweep < 64; ++sweep) {
        double off = a[0][1] * a[0][1] + a[0][2] * a[0][2] + a[1][2] * a[1][2];
        double scale = a[0][0] * a[0][0] + a[1][1] * a[1][1] + a[2][2] * a[2][2] + 2 * off;
        if (off <= 1e-36 * scale || off == 0.0) break;
        for (int p = 0; p < 2; ++p)
            for (int q = p + 1; q < 3; ++q) {
                double apq = a[p][q];
                if (apq == 0.0) continue;
                double theta = (a[q][q] - a[p][p]) / (2.0 * apq);
                double t = (theta >= 0 ? 1.0 : -1.0) / (std::abs(theta) + std::sqrt(theta * theta + 1.0));
                double c = 1.0 / std::sqrt(t * t + 1.0), s = t * c;
                for (int k = 0; k < 3; ++k) {  // A <- A J
                    double akp = a[k][p], akq = a[k][q];
                    a[k][p] = c * akp - s * akq;
                    a[k][q] = s * akp + c * akq;
                }
                for (int k = 0; k < 3; ++k) {  // A <- J^T A
                    double apk = a[p][k], aqk = a[q][k];
                    a[p][k] = c * apk - s * aqk;
                    a[q][k] = s * apk + c * aqk;
                }
                for (int k = 0; k < 3; ++k) {
                    double vkp = v[k][p], vkq = v[k][q];
                    v[k][p] = c * vkp - s * vkq;
                    v[k][q] = s * vkp + c * vkq;
                }
            }
    }
    int order[3] = {0, 1, 2};
    double d[3] = {a[0][0], a[1][1], a[2][2]};
    for (int i = 0; i < 3; ++i)
        for (int j = i + 1; j < 3; ++j)
            if (d[order[j]] < d[order[i]]) std::swap(order[i], order[j]);
    Eig3 e;
    for (int c = 0; c < 3; ++c) {
        e.val[c] = d[order[c]];
        for (int r = 0; r < 3; ++r) e.vec[r][c] = v[r][order[c]];
    }
    return e;
}

// ---------------------------------------------------------------------------
// Geometry::EigenDecompositionOfJcp (src/Geometry.cpp:27-69) + EigenDecomposition (:72-98).
void EigenDecompositionOfJcp(const Tube &t, const std::vector<V3> &subset_cpx, const std::vector<size_t> &set_from_subset,
                             const std::vector<int64_t> &subset_from_set, std::vector<Eig3> &out) {
    size_t ns = set_from_subset.size();
    std::vector<SpMat> Dc;
    BuildGradientMatrices(t, set_from_subset, subset_from_set, Dc);
    SpMat E;
    E.Resize(ns, ns);
    Interpolation interp(t, subset_cpx);
    interp.BuildInterpolationMatrix(t, subset_from_set, E);
    std::vector<std::vector<double>> cp(3, std::vector<double>(ns));
    for (size_t i = 0; i < ns; ++i)
        for (int d = 0; d < 3; ++d) cp[d][i] = subset_cpx[i][d];
    std::vector<double> J[3][3];
    std::vector<double> tmp;
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) {
            Dc[c].Multiply(cp[r], tmp);
            E.Multiply(tmp, J[r][c]);
        }
    out.resize(ns);
    for (size_t i = 0; i < ns; ++i) {
        double A[3][3], S[3][3];
        for (int r = 0; r < 3; ++r)
            for (int c = 0; c < 3; ++c) A[r][c] = J[r][c][i];
        for (int r = 0; r < 3; ++r)
            for (int c = 0; c < 3; ++c) S[r][c] = 0.5 * (A[r][c] + A[c][r]);
        out[i] = SymmetricEigen3(S);
    }
}

// Geometry::InterpolateUnorientedVectorFromNeighbours (src/Geometry.cpp:146-188).
void InterpolateUnorientedVectorFromNeighbours(const Tube &t, std::vector<V3> &vecs, const std::vector<size_t> &set_from_subset,
                                               const std::vector<int64_t> &subset_from_set, size_t i, double zero_tol) {
    V3 acc{0.0, 0.0, 0.0}, first{0, 0, 0};
    size_t num = 0;
    for (size_t nbr = 0; nbr < 6; ++nbr) {
        size_t index = set_from_subset[i];
        int64_t nb = t.neighbour((int64_t)index, nbr);
        if (nb >= 0) {
            int64_t sub = subset_from_set[nb];
            if (sub >= 0 && Norm(vecs[sub]) >= zero_tol) {
                if (num == 0) first = vecs[sub];
                if (Dot(first, vecs[sub]) > 0)
                    acc = Add(acc, vecs[sub]);
                else
                    acc = Sub(acc, vecs[sub]);
                ++num;
            }
        }
    }
    if (num > 0) vecs[i] = Div(acc, (double)num);
}

// Geometry::InterpolateUnorientedVectors (src/Geometry.cpp:205-236) +
// ApplyInterpolationToUnorientedVectors (:239-266): each row's first stencil
// vector fixes the orientation; later ones are added or subtracted by the sign
// of their dot product with it.
std::vector<V3> InterpolateUnorientedVectors(const Tube &t, const std::vector<int64_t> &subset_from_set, size_t subset_size,
                                             const std::vector<V3> &vecs, const std::vector<V3> &xq, bool normalize) {
    SpMat E;
    E.Resize(xq.size(), subset_size);
    Interpolation interp(t, xq);
    interp.BuildInterpolationMatrix(t, subset_from_set, E);
    std::vector<V3> vq(xq.size(), V3{0.0, 0.0, 0.0});
    for (size_t r = 0; r < E.rows; ++r) {
        V3 first{0.0, 0.0, 0.0};
        bool firstvisit = true;
        for (size_t e = E.ptr[r]; e < E.ptr[r + 1]; ++e) {
            const V3 &v = vecs[E.idx[e]];
            if (firstvisit) {
                first = v;
                firstvisit = false;
            }
            double dp = Dot(first, v);
            if (dp > 0.0)
                vq[r] = Add(vq[r], Scale(E.val[e], v));
            else
                vq[r] = Sub(vq[r], Scale(E.val[e], v));
        }
    }
    if (normalize)
        for (auto &v : vq) Normalize(v, 0.0);
    else
        for (auto &v : vq) v = Div(v, 64.0);
    return vq;
}

// Whole-tube surface normals: eigenvector 0 of the symmetrised Jcp
// (src/IBCSubset.cpp:192-228, use_Jcp_surface_normals branch).
std::vector<V3> NormalsFromJcp(const Tube &t) {
    std::vector<size_t> s2(t.nNodes());
    std::vector<int64_t> s1(t.nNodes());
    for (size_t i = 0; i < t.nNodes(); ++i) {
        s1[i] = (int64_t)i;
        s2[i] = i;
    }
    std::vector<Eig3> eig;
    EigenDecompositionOfJcp(t, t.cpx(), s2, s1, eig);
    std::vector<V3> n(t.nNodes());
    for (size_t i = 0; i < t.nNodes(); ++i)
        for (int d = 0; d < 3; ++d) n[i][d] = eig[i].vec[d][0];
    return n;
}

// Geometry::UnorientedSurfaceNormals (src/Geometry.cpp:101-126) with its defaults
// (normalised, zero_tol 1e-15): x - cp, interpolated from the neighbours where it
// vanishes, then Normalize (src/VectorMath.cpp:40-56: zero below the tolerance).
std::vector<V3> UnorientedSurfaceNormals(const Tube &t) {
    const size_t N = t.nNodes();
    std::vector<V3> n(N);
    for (size_t i = 0; i < N; ++i) n[i] = Sub(t.x()[i], t.cpx()[i]);
    std::vector<size_t> s2(N);
    std::vector<int64_t> s1(N);
    for (size_t i = 0; i < N; ++i) {
        s1[i] = (int64_t)i;
        s2[i] = i;
    }
    const double zero_tol = 1e-15;
    for (size_t i = 0; i < N; ++i)
        if (Norm(n[i]) < zero_tol) InterpolateUnorientedVectorFromNeighbours(t, n, s2, s1, i, zero_tol);
    for (size_t i = 0; i < N; ++i) {
        const double nn = Norm(n[i]);
        n[i] = nn > zero_tol ? Div(n[i], nn) : V3{0.0, 0.0, 0.0};
    }
    return n;
}

// ---------------------------------------------------------------------------
// IBCSubset (src/IBCSubset.cpp:12-268)

void IBCSubset::ComputeSubset(const Surface &ibc, const Tube &t, const std::vector<V3> &normals_on_tube) {
    m_meta = ibc.spec().meta;
    ComputeSubsetNearIBC(ibc, t);
    m_subset_from_set.assign(t.nNodes(), -1);
    for (size_t i = 0; i < m_set_from_subset.size(); ++i) m_subset_from_set[m_set_from_subset[i]] = (int64_t)i;
    ComputeCPdiff(ibc, t);
    if (m_meta.use_cp_diff_directions)
        m_directions = m_cp_diff;
    else
        ComputeFrameBasedDirections(t, normals_on_tube);
}

// ComputeSubsetNearIBC (:39-109): BFS over tube neighbours from the tube node
// nearest xp[0] of the IBC; a node is kept iff its IBC distance < 2r.  The
// start node itself is only added when it is reached again as a neighbour.
void IBCSubset::ComputeSubsetNearIBC(const Surface &ibc, const Tube &t) {
    double radius = 2.0 * t.TubeRadius();
    int64_t start = t.NearestTubeIndex(ibc.xp()[0]);
    if (start < 0) throw std::runtime_error("IBCSubset: IBC start point is not near the tube");
    std::vector<size_t> queue{(size_t)start};
    std::vector<bool> visited(t.nNodes(), false);
    size_t head = 0;
    V3 cp;
    double dist;
    size_t bdy;
    while (head < queue.size()) {
        size_t cur = queue[head];
        for (size_t nbr = 0; nbr < 6; ++nbr) {
            int64_t nb = t.neighbour((int64_t)cur, nbr);
            if (nb >= 0 && !visited[nb]) {
                visited[nb] = true;
                ibc.ClosestPoint(t.x()[nb], cp, dist, bdy);
                if (dist < radius) {
                    m_cpx_c.push_back(cp);
                    m_dist_c.push_back(dist);
                    m_bdy.push_back(bdy);
                    m_set_from_subset.push_back((size_t)nb);
                    queue.push_back((size_t)nb);
                }
            }
        }
        head++;
    }
}

// ComputeCPdiff (:156-187) including the S-perp fix-up from neighbours.
void IBCSubset::ComputeCPdiff(const Surface &ibc, const Tube &t) {
    m_cp_diff.assign(size(), V3{0, 0, 0});
    for (size_t i = 0; i < size(); ++i) {
        if (m_bdy[i] > 0 && m_meta.use_cp_diff_directions) {
            V3 proj = Sub(Scale(2.0, m_cpx_c[i]), t.x()[m_set_from_subset[i]]);
            V3 cps, cpc;
            t.ClosestPoint(proj, cps);
            ibc.ClosestPoint(proj, cpc);
            m_cp_diff[i] = Sub(cpc, cps);
        } else {
            m_cp_diff[i] = Sub(t.cpx()[m_set_from_subset[i]], m_cpx_c[i]);
        }
    }
    for (size_t i = 0; i < size(); ++i)
        if (Norm(m_cp_diff[i]) < m_meta.on_ibc_tolerance)
            InterpolateUnorientedVectorFromNeighbours(t, m_cp_diff, m_set_from_subset, m_subset_from_set, i, m_meta.on_ibc_tolerance);
}

// ComputeFrameBasedDirections, 3-D branch (:190-268).
void IBCSubset::ComputeFrameBasedDirections(const Tube &t, const std::vector<V3> &normals_on_tube) {
    m_normals_tube = normals_on_tube;
    m_normals = InterpolateUnorientedVectors(t, [&]() {
        std::vector<int64_t> id(t.nNodes());
        for (size_t i = 0; i < t.nNodes(); ++i) id[i] = (int64_t)i;
        return id;
    }(), t.nNodes(), m_normals_tube, m_cpx_c, true);
    m_binormals.assign(size(), V3{0, 0, 0});
    m_directions.assign(size(), V3{0, 0, 0});
    std::vector<Eig3> eig;
    EigenDecompositionOfJcp(t, m_cpx_c, m_set_from_subset, m_subset_from_set, eig);
    m_tangents.assign(size(), V3{0.0, 0.0, 0.0});
    for (size_t i = 0; i < size(); ++i) {
        if (std::abs(eig[i].val[2]) < 1e-8) {  // a point IBC: J_cp_C vanishes
            m_binormals[i] = V3{0.0, 0.0, 0.0};
            m_directions[i] = Sub(m_cp_diff[i], Scale(Dot(m_normals[i], m_cp_diff[i]), m_normals[i]));
        } else {
            for (int d = 0; d < 3; ++d) m_tangents[i][d] = eig[i].vec[d][2];
            m_binormals[i] = Cross(m_tangents[i], m_normals[i]);
            m_directions[i] = Scale(Dot(m_binormals[i], m_cp_diff[i]), m_binormals[i]);
        }
    }
}

// ---------------------------------------------------------------------------
// IBCDOFSubset (src/IBCDOFSubset.cpp:10-227)

void IBCDOFSubset::ComputeDOFSubset(const Surface &ibc, const IBCSubset &sub, const Tube &t) {
    m_meta = sub.meta();
    const double rad = m_meta.ibc_DOFSubset_radius_scale * t.TubeRadius();
    for (size_t i = 0; i < sub.size(); ++i) {
        if (sub.dist()[i] < rad) {
            m_set_from_subset.push_back(sub.SetIndexFromSubsetIndex()[i]);
            m_cpx_c.push_back(sub.cpx()[i]);
            m_cp_diff.push_back(sub.cp_diff()[i]);
            m_dist_c.push_back(sub.dist()[i]);
            m_bdy.push_back(sub.bdy()[i]);
        }
    }
    m_subset_from_set.assign(t.nNodes(), -1);
    for (size_t i = 0; i < size(); ++i) m_subset_from_set[m_set_from_subset[i]] = (int64_t)i;
    if (m_meta.use_cp_diff_directions) {
        m_directions = m_cp_diff;
    } else {
        for (size_t i = 0; i < sub.size(); ++i)
            if (sub.dist()[i] < rad) {
                m_normals.push_back(sub.surface_normals()[i]);
                m_tangents.push_back(sub.tangents()[i]);
                m_binormals.push_back(sub.binormals()[i]);
                m_directions.push_back(sub.directions()[i]);
            }
    }
    m_which_side.assign(size(), 0);
    if (m_meta.is_oriented) OrientSubset(ibc, t);

    if ((m_meta.boundary_type[0] == 0 || m_meta.boundary_type[1] == 0) && m_meta.boundary_order == 2) {
        for (size_t i = 0; i < size(); ++i) {
            size_t bc = m_meta.is_oriented ? m_which_side[i] - 1 : 0;
            if (m_meta.boundary_type[bc] == 0) m_dir_set_from_subset.push_back(i);
        }
        m_dir_subset_from_set.assign(size(), -1);
        for (size_t i = 0; i < m_dir_set_from_subset.size(); ++i) m_dir_subset_from_set[m_dir_set_from_subset[i]] = (int64_t)i;
    }
    if (m_meta.boundary_order == 2) {
        m_cp_bar.assign(size(), V3{0, 0, 0});
        for (size_t i = 0; i < size(); ++i) {
            V3 proj = Sub(Scale(2.0, m_cpx_c[i]), t.x()[m_set_from_subset[i]]);
            t.ClosestPoint(proj, m_cp_bar[i]);
        }
    }
    // ComputeExtensionMatrix (:110-125)
    const std::vector<V3> &xq = (m_meta.boundary_order == 2) ? m_cp_bar : m_cpx_c;
    Interpolation interp(t, xq);
    m_E.Resize(size(), t.nNodes());
    interp.BuildInterpolationMatrix(t, m_E);
}

// OrientSubset (:128-227): BFS over the DOF subset propagating which_side by the
// sign of neighbouring directions, then flipped so point_on_side1 is side 1.
void IBCDOFSubset::OrientSubset(const Surface &ibc, const Tube &t) {
    size_t start = 0;
    for (size_t i = 0; i < size(); ++i)
        if (Norm(m_directions[i]) >= m_meta.on_ibc_tolerance) {
            start = i;
            break;
        }
    m_which_side[start] = 1;
    std::vector<size_t> queue{start};
    std::vector<bool> visited(size(), false);
    size_t head = 0;
    while (head < queue.size()) {
        size_t f = queue[head];
        if (!visited[f]) {
            size_t s = m_set_from_subset[f];
            visited[f] = true;
            for (size_t nbr = 0; nbr < 6; ++nbr) {
                int64_t nb = t.neighbour((int64_t)s, nbr);
                if (nb < 0) continue;
                int64_t ns = m_subset_from_set[nb];
                if (ns >= 0) {
                    if (m_which_side[ns] == 0) {
                        if (Dot(m_directions[f], m_directions[ns]) < 0)
                            m_which_side[ns] = (m_which_side[f] == 1) ? 2 : 1;
                        else
                            m_which_side[ns] = m_which_side[f];
                    }
                    queue.push_back((size_t)ns);
                }
            }
        }
        head++;
    }
    if (m_meta.point_on_side1.size() == 3) {
        V3 ps{m_meta.point_on_side1[0], m_meta.point_on_side1[1], m_meta.point_on_side1[2]};
        size_t nearest = 0;
        double nd = std::numeric_limits<double>::max();
        for (size_t i = 0; i < size(); ++i) {
            double dd = Distance(ps, t.x()[m_set_from_subset[i]]);
            V3 cpc;
            ibc.ClosestPoint(ps, cpc);
            V3 cpd = Sub(ps, cpc);
            if (dd < nd && Norm(m_cp_diff[i]) >= 2 * t.dx() && Dot(cpd, m_cp_diff[i]) > 0) {
                nd = dd;
                nearest = i;
            }
        }
        if (m_which_side[nearest] == 1)
            for (auto &w : m_which_side) w = (w == 1) ? 2 : (w == 2 ? 1 : w);
    }
}

// ---------------------------------------------------------------------------
// IBCSubsets (src/IBCSubsets.cpp:11-116)

void IBCSubsets::Initialize(const Tube &t, const std::vector<SurfaceSpec> &specs) {
    m_num = specs.size();
    m_surf.clear();
    for (const auto &s : specs) m_surf.emplace_back(s);
    std::vector<V3> normals;
    // the surface normals on the tube each IBC's frames use (IBCSubset::ComputeFrameBasedDirections,
    // src/IBCSubset.cpp:190-215): Jcp eigenvectors, or x - cp when use_Jcp_surface_normals is off
    std::vector<V3> normals_x;
    bool need = false, need_x = false;
    for (const auto &s : specs)
        if (!s.meta.use_cp_diff_directions) (s.meta.use_Jcp_surface_normals ? need : need_x) = true;
    if (need) normals = NormalsFromJcp(t);
    if (need_x) normals_x = UnorientedSurfaceNormals(t);
    m_tag.assign(m_num, IBCSubset());
    for (size_t c = 0; c < m_num; ++c)
        m_tag[c].ComputeSubset(m_surf[c], t, specs[c].meta.use_Jcp_surface_normals ? normals : normals_x);
    m_dof.assign(m_num, IBCDOFSubset());
    for (size_t c = 0; c < m_num; ++c) m_dof[c].ComputeDOFSubset(m_surf[c], m_tag[c], t);
    // IBCStartingColumns (:74-94)
    m_start.assign(m_num, 0);
    m_dstart.assign(m_num, 0);
    if (m_num > 0) {
        m_start[0] = t.nNodes();
        m_dstart[0] = t.nNodes();
    }
    for (size_t c = 1; c < m_num; ++c) {
        m_start[c] = m_start[c - 1] + m_dof[c - 1].size();
        const IBCMeta &mc = meta(c);
        if ((mc.boundary_type[0] == 0 || mc.boundary_type[1] == 0) && mc.boundary_order == 2)
            m_dstart[c] = m_dstart[c - 1] + m_dof[c - 1].DirichletSetIndexFromSubsetIndex().size();
    }
    // TotalDOFs (:97-116)
    m_id_start = 0;
    m_num2 = 0;
    m_total = 0;
    for (size_t c = 0; c < m_num; ++c) {
        const IBCMeta &mc = meta(c);
        if ((mc.boundary_type[0] == 0 || mc.boundary_type[1] == 0) && mc.boundary_order == 2) {
            m_id_start += 1;
            m_num2 += m_dof[c].DirichletSetIndexFromSubsetIndex().size();
        }
        m_total += m_dof[c].size();
    }
    if (m_id_start != 0) m_id_start = m_total;
}

size_t DirichletValueRow(const IBCSubsets &ibc, size_t c, size_t i) {
    if (ibc.meta(c).boundary_order == 2)
        return ibc.IdentityRowsStart() + (size_t)ibc.DOFSubset()[c].DirichletSubsetIndexFromSetIndex()[i] + ibc.DirichletIBCColumnStartIndex(c);
    return ibc.IdentityRowsStart() + i + ibc.IBCColumnStartIndex(c);
}

std::vector<bool> IBCIdentityRows(const Tube &t, const IBCSubsets &ibc) {
    std::vector<bool> id(t.nNodes() + ibc.TotalIBCDOFs() + ibc.Num2ndOrderDirichletRows(), false);
    for (size_t c = 0; c < ibc.NumIBCs(); ++c)
        for (size_t i = 0; i < ibc.DOFSubset()[c].size(); ++i) {
            size_t bc = ibc.meta(c).is_oriented ? ibc.DOFSubset()[c].which_side()[i] - 1 : 0;
            if (ibc.meta(c).boundary_type[bc] == 0) id[DirichletValueRow(ibc, c, i)] = true;
        }
    return id;
}

// ---------------------------------------------------------------------------
// IBCMatrixManipulations (src/IBCMatrixManipulations.cpp)

// TagStencils (:424-463).
std::vector<uint8_t> TagStencils(const SpMat &A, const Tube &t, const IBCSubsets &ibc, const std::vector<V3> &dirs,
                                 const std::vector<int64_t> &dsub, size_t c, double flip) {
    (void)t;
    const IBCSubset &ts = ibc.TaggingSubset()[c];
    std::vector<uint8_t> tags(A.nnz(), 1);
    for (size_t r = 0; r < A.rows; ++r)
        for (size_t e = A.ptr[r]; e < A.ptr[r + 1]; ++e) {
            int64_t di = dsub[r];
            int64_t sp = ts.SubsetIndexFromSetIndex()[A.idx[e]];
            if (di >= 0 && sp >= 0 && ts.bdy()[sp] == 0) {
                double dp = flip * Dot(dirs[di], ts.directions()[sp]);
                if (dp < 0.0) tags[e] = 2;
            }
        }
    return tags;
}

// MoveToIBCColumns (:189-216).
static void MoveToIBCColumns(const SpMat &A, const std::vector<std::vector<uint8_t>> &tags, const IBCSubsets &ibc,
                             std::vector<Triplet> &coeffs) {
    for (size_t r = 0; r < A.rows; ++r)
        for (size_t e = A.ptr[r]; e < A.ptr[r + 1]; ++e) {
            size_t cnt = 0;
            for (size_t c = 0; c < ibc.NumIBCs(); ++c) {
                int64_t s = ibc.DOFSubset()[c].SubsetIndexFromSetIndex()[A.idx[e]];
                if (tags[c][e] == 2 && s >= 0) {
                    ++cnt;
                    coeffs.push_back({r, (size_t)s + ibc.IBCColumnStartIndex(c), A.val[e]});
                }
            }
            if (cnt == 0) coeffs.push_back({r, A.idx[e], A.val[e]});
        }
}

// AddFiniteDifferenceIBCRows (:219-251).
static void AddFiniteDifferenceIBCRows(const SpMat &A, const std::vector<std::vector<uint8_t>> &tags, const IBCSubsets &ibc,
                                       std::vector<Triplet> &coeffs) {
    for (size_t r = 0; r < A.rows; ++r)
        for (size_t e = A.ptr[r]; e < A.ptr[r + 1]; ++e)
            for (size_t c = 0; c < ibc.NumIBCs(); ++c) {
                const auto &sub = ibc.DOFSubset()[c].SubsetIndexFromSetIndex();
                size_t st = ibc.IBCColumnStartIndex(c);
                if (tags[c][e] == 2 && sub[r] >= 0) {
                    coeffs.push_back({(size_t)sub[r] + st, A.idx[e], A.val[e]});
                } else if (sub[r] >= 0 && sub[A.idx[e]] >= 0) {
                    coeffs.push_back({(size_t)sub[r] + st, (size_t)sub[A.idx[e]] + st, A.val[e]});
                }
            }
}

// AddIBCFiniteDifference (:38-71).
SpMat AddIBCFiniteDifference(const SpMat &L, const Tube &t, const IBCSubsets &ibc) {
    std::vector<std::vector<uint8_t>> tags(ibc.NumIBCs());
    for (size_t c = 0; c < ibc.NumIBCs(); ++c)
        tags[c] = TagStencils(L, t, ibc, ibc.TaggingSubset()[c].directions(), ibc.TaggingSubset()[c].SubsetIndexFromSetIndex(), c);
    std::vector<Triplet> coeffs;
    MoveToIBCColumns(L, tags, ibc, coeffs);
    AddFiniteDifferenceIBCRows(L, tags, ibc, coeffs);
    for (size_t c = 0; c < ibc.NumIBCs(); ++c)
        for (size_t i = 0; i < ibc.DOFSubset()[c].size(); ++i) {
            size_t bc = ibc.meta(c).is_oriented ? ibc.DOFSubset()[c].which_side()[i] - 1 : 0;
            if (ibc.meta(c).boundary_type[bc] == 0 && ibc.meta(c).boundary_order == 2) {
                size_t r = DirichletValueRow(ibc, c, i);
                coeffs.push_back({r, r, 1.0});
            }
        }
    size_t n = L.rows + ibc.TotalIBCDOFs() + ibc.Num2ndOrderDirichletRows();
    SpMat out;
    out.FromTriplets(n, L.cols + ibc.TotalIBCDOFs() + ibc.Num2ndOrderDirichletRows(), coeffs);
    return out;
}

// AddExtensionIBCRows (:118-186).
static void AddExtensionIBCRows(const Tube &t, const IBCSubsets &ibc, std::vector<Triplet> &coeffs) {
    for (size_t c = 0; c < ibc.NumIBCs(); ++c) {
        const IBCDOFSubset &dof = ibc.DOFSubset()[c];
        const IBCMeta &mc = ibc.meta(c);
        const SpMat &Ei = dof.cpExtensionMatrix();
        std::vector<int64_t> ident(dof.size());
        for (size_t i = 0; i < dof.size(); ++i) ident[i] = (int64_t)i;
        std::vector<uint8_t> tg = TagStencils(Ei, t, ibc, dof.directions(), ident, c, -1.0);
        size_t st = ibc.IBCColumnStartIndex(c);
        for (size_t r = 0; r < Ei.rows; ++r)
            for (size_t e = Ei.ptr[r]; e < Ei.ptr[r + 1]; ++e) {
                size_t bc = mc.is_oriented ? dof.which_side()[r] - 1 : 0;
                double scale = (mc.boundary_type[bc] == 0) ? -1.0 : 1.0;
                if (mc.boundary_type[bc] == 1 || (mc.boundary_type[bc] == 0 && mc.boundary_order == 2)) {
                    int64_t s = dof.SubsetIndexFromSetIndex()[Ei.idx[e]];
                    if (tg[e] == 2 && s >= 0)
                        coeffs.push_back({r + st, (size_t)s + st, scale * Ei.val[e]});
                    else
                        coeffs.push_back({r + st, Ei.idx[e], scale * Ei.val[e]});
                }
            }
        if (mc.boundary_order == 2) {
            for (size_t i = 0; i < dof.size(); ++i) {
                size_t bc = mc.is_oriented ? dof.which_side()[i] - 1 : 0;
                if (mc.boundary_type[bc] == 0) coeffs.push_back({i + st, DirichletValueRow(ibc, c, i), 2.0});
            }
            for (size_t i = 0; i < dof.size(); ++i) {
                size_t bc = mc.is_oriented ? dof.which_side()[i] - 1 : 0;
                if (mc.boundary_type[bc] == 0) {
                    size_t r = DirichletValueRow(ibc, c, i);
                    coeffs.push_back({r, r, 1.0});
                }
            }
        } else {
            for (size_t i = 0; i < dof.size(); ++i) {
                size_t bc = mc.is_oriented ? dof.which_side()[i] - 1 : 0;
                if (mc.boundary_type[bc] == 0) {
                    size_t r = ibc.IdentityRowsStart() + i + st;
                    coeffs.push_back({r, r, 1.0});
                }
            }
        }
    }
}

// AddIBCExtension (:12-35).
SpMat AddIBCExtension(const SpMat &E, const Tube &t, const IBCSubsets &ibc) {
    std::vector<std::vector<uint8_t>> tags(ibc.NumIBCs());
    for (size_t c = 0; c < ibc.NumIBCs(); ++c)
        tags[c] = TagStencils(E, t, ibc, ibc.TaggingSubset()[c].directions(), ibc.TaggingSubset()[c].SubsetIndexFromSetIndex(), c);
    std::vector<Triplet> coeffs;
    MoveToIBCColumns(E, tags, ibc, coeffs);
    AddExtensionIBCRows(t, ibc, coeffs);
    size_t extra = ibc.TotalIBCDOFs() + ibc.Num2ndOrderDirichletRows();
    SpMat out;
    out.FromTriplets(E.rows + extra, E.cols + extra, coeffs);
    return out;
}

// PlotPointsCPDiff (:254-416), non-oriented part, and AddIBCPlotInterpolation (:84-106).
SpMat AddIBCPlotInterpolation(const SpMat &plotE, const Tube &t, const IBCSubsets &ibc) {
    const std::vector<V3> &xp = t.surface().xp();
    std::vector<std::vector<uint8_t>> tags(ibc.NumIBCs());
    for (size_t c = 0; c < ibc.NumIBCs(); ++c) {
        const IBCSubset &ts = ibc.TaggingSubset()[c];
        std::vector<V3> scp, sdiff;
        std::vector<size_t> sbdy, set_from_sub;
        std::vector<int64_t> sub_from_set(xp.size(), -1);
        size_t count = 0;
        for (size_t i = 0; i < xp.size(); ++i) {
            V3 cpc;
            double dummy;
            size_t bdy;
            ibc.ClosestPoint(c, xp[i], cpc, dummy, bdy);
            V3 cd = Sub(xp[i], cpc);
            if (Norm(cd) < 2.0 * t.TubeRadius()) {
                scp.push_back(cpc);
                sdiff.push_back(cd);
                sbdy.push_back(bdy);
                sub_from_set[i] = (int64_t)count;
                set_from_sub.push_back(i);
                ++count;
            }
        }
        for (size_t i = 0; i < count; ++i)
            if (Norm(sdiff[i]) < ibc.meta(c).on_ibc_tolerance) {
                int64_t nearest = t.NearestTubeIndex(xp[set_from_sub[i]]);
                if (nearest >= 0 && ts.SubsetIndexFromSetIndex()[nearest] >= 0)
                    sdiff[i] = ts.cp_diff()[ts.SubsetIndexFromSetIndex()[nearest]];
            }
        std::vector<V3> dirs(count, V3{0, 0, 0});
        if (ibc.meta(c).use_cp_diff_directions) {
            for (size_t i = 0; i < count; ++i) {
                if (sbdy[i] > 0) {
                    V3 proj = Sub(Scale(2.0, scp[i]), xp[set_from_sub[i]]);
                    V3 cps, cpc;
                    t.ClosestPoint(proj, cps);
                    double d;
                    size_t b;
                    ibc.ClosestPoint(c, proj, cpc, d, b);
                    sdiff[i] = Sub(cpc, cps);
                }
                dirs[i] = sdiff[i];
            }
        } else {
            std::vector<V3> bn = InterpolateUnorientedVectors(t, ts.SubsetIndexFromSetIndex(), ts.size(), ts.binormals(), scp, true);
            for (size_t i = 0; i < count; ++i) dirs[i] = Scale(Dot(bn[i], sdiff[i]), bn[i]);
        }
        tags[c] = TagStencils(plotE, t, ibc, dirs, sub_from_set, c);
    }
    std::vector<Triplet> coeffs;
    MoveToIBCColumns(plotE, tags, ibc, coeffs);
    SpMat out;
    out.FromTriplets(plotE.rows, plotE.cols + ibc.TotalIBCDOFs() + ibc.Num2ndOrderDirichletRows(), coeffs);
    return out;
}

}  // namespace cpmref
