/*
 * cpm_gpu.h — C-ABI of the GB300-native closest-point-method solve path.
 *
 * The entry points replace the reference's BUILD_CUSTOM_SOLVER path
 * (nathandking/cpm-ibc).  Every declaration names the reference interface it
 * stands in for.  Plain pointers and sizes only; host buffers are caller-owned
 * and copied in/out; device state is owned by opaque handles.  All functions
 * return 0 on success or a negative cpm_status; cpm_last_error() describes the
 * last failure of the calling thread.
 */
#ifndef CPM_GPU_H
#define CPM_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes.  The reference throws std::runtime_error for a base point
 * outside the tube (src/Tube.cpp:477-480) and for unknown surfaces
 * (src/Surface.cpp:188), and silently returns after 100000 BiCGStab
 * iterations (src/BiCGStab.h:107); here each is a status. */
enum cpm_status {
    CPM_OK = 0,
    CPM_ERR_INVALID_ARG = -1,
    CPM_ERR_CUDA = -2,
    CPM_ERR_OOM = -3,
    CPM_ERR_BASEPOINT_OUTSIDE_TUBE = -4,
    CPM_ERR_NOT_CONVERGED = -5,
    CPM_ERR_BREAKDOWN = -6,
    CPM_ERR_UNSUPPORTED = -7,
    CPM_ERR_ADMISSION = -8,
    CPM_ERR_TIMEOUT = -9
};

/* Surface kinds: the reference dispatches on a name string
 * (src/Surface.cpp:61-190); the in-scope kinds are numbered. */
enum cpm_surface_kind {
    CPM_SPHERE = 0,        /* cpSphere    src/Surface.cpp:710-741  params R [, centre] */
    CPM_TORUS = 1,         /* cpTorus     src/Surface.cpp:800-838  params R, r          */
    CPM_CIRCLE3D = 2,      /* cpCircle3D  src/Surface.cpp:464-504  params R, centre, normal */
    CPM_POINT = 3,         /* cpPoint     src/Surface.cpp:840-848  params x, y, z       */
    CPM_TRIANGULATION = 4, /* cpTri       src/Surface.cpp:1751-1780 (fcpw in the reference) */
    CPM_POLYLINE = 5       /* cpTri on line segments, same lines                          */
};

/* SurfaceSpecifier (src/SurfaceSpecifier.h:198-216) + IBCMetaData
 * (src/IBCMetaData.h:9-24) in one plain struct. */
typedef struct cpm_surface_desc {
    int32_t kind;
    int32_t nparams;
    double params[8];
    double bbox[2];
    int64_t nverts;
    const double *verts;   /* 3*nverts, host memory */
    int64_t nprims;
    const int64_t *prims;  /* 3*nprims triangles or 2*nprims segments */
    int32_t boundary_order;         /* IBCMetaData::boundary_order (1 or 2) */
    int32_t boundary_type[2];       /* 0 Dirichlet, 1 Neumann */
    int32_t is_oriented;
    int32_t has_point_on_side1;
    int32_t use_cp_diff_directions;
    int32_t use_Jcp_surface_normals;
    int32_t pad0;
    double on_ibc_tolerance;
    double point_on_side1[3];
    double dof_radius_scale;        /* IBCMetaData::ibc_DOFSubset_radius_scale */
} cpm_surface_desc;

typedef struct cpm_tube_s *cpm_tube_t;
typedef struct cpm_opset_s *cpm_opset_t;
typedef struct cpm_solver_s *cpm_solver_t;

typedef struct cpm_tube_info {
    int64_t n_nodes;     /* Tube::nNodes            src/Tube.h:51 */
    int64_t n1d;         /* Tube::N1d               src/Tube.h:54 */
    int64_t n_bricks;    /* occupied 4^3 bricks */
    int64_t n_visited;   /* grid nodes whose closest point was evaluated */
    double dx;           /* Tube::dx */
    double xstart;       /* Tube::xstart()[d] (equal in every dimension) */
    double radius;       /* Tube::TubeRadius        src/Tube.cpp:131-138 */
    int32_t p;           /* interpolation degree */
    int32_t pad;
} cpm_tube_info;

/* ---- errors / device ---------------------------------------------------- */
const char *cpm_last_error(void);
/* Select the CUDA device for this process's library state; call before any
 * other entry point (the library stream is created on the current device). */
int cpm_set_device(int32_t device);
int cpm_device_info(char *name, int64_t name_len, int64_t *free_bytes, int64_t *total_bytes, int32_t *sm_count);

/* ---- Tube ----------------------------------------------------------------
 * Tube(SurfaceSpecifier&, size_t p, Scalar dx)  src/Tube.h:45, src/Tube.cpp:46-55,295-461.
 * Builds the band on the device: analytic (or mesh) closest points, band test
 * |dist| <= r, 6-connected component of the seed node, Morton-ordered 4^3
 * bricks, neighbour / brick tables, base points and tricubic weights. */
int cpm_tube_build(const cpm_surface_desc *surface, int32_t p, double dx, cpm_tube_t *out);

/* Same tube, but the closest point and distance of every grid node the build
 * evaluates come from the caller (keys = grid linear indices i*N1d^2+j*N1d+k,
 * sorted ascending).  "Given the same closest points" parity entry point. */
int cpm_tube_build_from_cp(const cpm_surface_desc *surface, int32_t p, double dx, int64_t n, const int64_t *keys,
                           const double *cp, const double *dist, cpm_tube_t *out);

int cpm_tube_info_get(cpm_tube_t t, cpm_tube_info *info);

/* Tube accessors, exported in device (Morton-brick) order together with each
 * node's grid linear index `rec` (Node::recIndex, src/Node.h:11), so callers
 * can permute to the reference's BFS order.  Any pointer may be NULL.
 *   x, cp: 3*n; dist: n; bpt_rec: n (grid linear index of the base point,
 *   Tube::bpt src/Tube.h:147 as a grid index); nbr: 6*n tube indices or -1
 *   (Node::neighbour order +x,-x,+y,-y,+z,-z, src/Node.h:23);
 *   w: 12*n tricubic 1-D weights [d][j] (Interpolation m_w, src/Interpolation.h:29). */
int cpm_tube_export(cpm_tube_t t, int64_t *rec, double *x, double *cp, double *dist, int64_t *bpt_rec, int64_t *nbr,
                    double *w);

/* Tube node numbering of the reference: order[i] is the device index of the
 * node the reference's breadth-first flood numbers i (Tube::BuildTube,
 * src/Tube.cpp:321-454; seed first, neighbours +x,-x,+y,-y,+z,-z), so that
 * device-ordered exports can be permuted into reference-shaped vectors. */
int cpm_tube_reference_order(cpm_tube_t t, int64_t *order);

/* Interpolation(Tube&, xq) + BuildInterpolationMatrix (src/Interpolation.cpp:23-36,52-121):
 * per query point the 64 column indices (device tube order) and E entries
 * (w2[k]*w1[j]*w0[i], walk +x outer, +y, +z inner).  Returns
 * CPM_ERR_BASEPOINT_OUTSIDE_TUBE like Tube::ComputeBasePoints. */
int cpm_interp_query(cpm_tube_t t, int64_t n, const double *xq, int64_t *cols, double *vals);

/* Tube::NearestTubeIndex (src/Tube.h:116-121): per point x[3i..3i+2] the device
 * index of the tube node at the nearest grid point, or -1 where that grid point
 * is not in the tube. */
int cpm_tube_nearest(cpm_tube_t t, int64_t n, const double *x, int64_t *idx);

/* Surface::xp() of an IBC curve (Surface::GetSurfaceParameterization,
 * src/Surface.cpp:194-216, paramCircle3D :1883-1904): a Circle3D's 100 points at
 * theta_i = i 2 pi / 99, a Point, or a polyline's vertices.  *n is the capacity
 * of xp on input and the count on output; xp = NULL queries the count. */
int cpm_ibc_plot_points(const cpm_surface_desc *ibc, int64_t *n, double *xp);

/* Surface::ClosestPoint(x, cpx, dist, bdy) (src/Surface.h:33-34, src/Surface.cpp:61-190) for
 * n points x (3n doubles) of any surface kind: cp (3n) and dist (n) as the reference's
 * closest-point functions give them.  max_dist > 0 bounds the triangle-mesh and polyline
 * searches: a point farther than max_dist from every primitive reports dist > max_dist and an
 * unspecified cp; max_dist <= 0 searches every primitive.  bdy is not reported.  This is the
 * query the reference's callers use to pick constraint nodes against curves
 * (examples/GeodesicDistanceBeetle/GeodesicDistanceBeetle.cpp:36-52). */
int cpm_closest_points(const cpm_surface_desc *surface, int64_t n, const double *x, double max_dist, double *cp,
                       double *dist);

int cpm_tube_destroy(cpm_tube_t t);

/* ---- Operator set (Lfull, Efull, identity rows) -------------------------
 * Helpers::SetupMatrices (src/Helpers.cpp:86-93), IBCSubsets::Initialize
 * (src/IBCSubsets.h:23) and IBCMatrixManipulations::AddIBCFiniteDifference /
 * AddIBCExtension (src/IBCMatrixManipulations.cpp:12-71) as one object whose
 * rows are: tube rows (device order), then IBC DOF rows and Dirichlet value
 * rows in the reference's column layout (src/IBCSubsets.cpp:74-116).  A stencil
 * entry that lies across several IBCs moves to each of their DOF columns, as
 * MoveToIBCColumns keeps it (src/IBCMatrixManipulations.cpp:189-216).
 * CPM_ERR_UNSUPPORTED for IBCs of different boundary orders in one set (the
 * reference's identity-row numbering has no place for an order-1 IBC's rows once
 * another IBC is of order 2). */
int cpm_opset_create(cpm_tube_t t, int32_t n_ibc, const cpm_surface_desc *ibcs, cpm_opset_t *out);

/* Closest points computed by the caller: n query points x (3n), their closest
 * points cp (3n) and distances dist (n, or NULL).  A point is matched by the
 * exact bits of its three coordinates. */
typedef struct cpm_cp_table {
    int64_t n;
    const double *x;
    const double *cp;
    const double *dist;
} cpm_cp_table;

/* cpm_opset_create "given the same closest points", the operator-set
 * counterpart of cpm_tube_build_from_cp.  IBCSubset::ComputeSubsetNearIBC
 * (src/IBCSubset.cpp:39-109) takes IBC c's closest point and distance at a
 * tube node's grid coordinates from ibc_cp[c], and IBCDOFSubset's cp-bar
 * (src/IBCDOFSubset.cpp:63-73) takes the surface's closest point at the
 * projection 2 cp_c - x from surface_cp.  Points a table lacks (and a NULL
 * table) keep the device's own closest points.  The tables are copied; later
 * evaluation queries (cpm_opset_plot_interp) use them too. */
int cpm_opset_create_from_cp(cpm_tube_t t, int32_t n_ibc, const cpm_surface_desc *ibcs, const cpm_cp_table *ibc_cp,
                             const cpm_cp_table *surface_cp, cpm_opset_t *out);

/* sizes (9 entries): [D, N, total_ibc_dofs, num_2nd_order_rows, n_ibc, n_patched_rows,
 * n_moved_entries, rows whose E row is patched, moved E stencil points] */
int cpm_opset_sizes(cpm_opset_t op, int64_t *sizes);

/* Row layout for right-hand sides (PoissonWithIBC::GetRHS, problems/PoissonWithIBC.cpp:92-133):
 * kind 0 tube row (f at its closest point), 1 IBC DOF row (f at the DOF's IBC
 * closest point), 2 Dirichlet value row (IBC value), 3 other.  point: 3*D. */
int cpm_opset_rows(cpm_opset_t op, uint8_t *identity, int32_t *kind, int32_t *ibc, double *point);

/* Side of the curve of every row (IBCDOFSubset::which_side, src/IBCDOFSubset.cpp:128-227):
 * 1 or 2 on an IBC's DOF and Dirichlet value rows (always 1 unless the IBC is
 * oriented), 0 on other rows.  PoissonWithIBC::GetRHS passes it to the boundary
 * value function (problems/PoissonWithIBC.cpp:92-133). */
int cpm_opset_row_sides(cpm_opset_t op, int32_t *side);

/* IBC subsets of IBC c (IBCSubset / IBCDOFSubset, src/IBCSubset.h, src/IBCDOFSubset.h):
 * sizes [tagging, dof, column start, dirichlet column start, identity rows start]
 * and the subsets as device tube indices in the reference's BFS order. */
int cpm_opset_ibc_sizes(cpm_opset_t op, int32_t c, int64_t *sizes);
int cpm_opset_ibc_export(cpm_opset_t op, int32_t c, int64_t *tag_set, int64_t *dof_set, double *dof_cp);

/* Assembled Lfull / Efull (which = 0 / 1), or the gradient matrices Dc_x, Dc_y,
 * Dc_z of the tube rows (which = 5, 6, 7; FDMatrices::BuildGradientMatrices,
 * src/FDMatrices.cpp:66-92; rows past the tube empty) as CSR in device row/column
 * order, for oracle comparison (columns sorted ascending). nnz query with ptr = NULL. */
int cpm_opset_export_csr(cpm_opset_t op, int32_t which, int64_t *nnz, int64_t *ptr, int64_t *idx, double *val);

/* Evaluation of a solution at surface points (replaces Helpers::GetPlotInterpMatrix
 * + IBCMatrixManipulations::AddIBCPlotInterpolation, src/Helpers.cpp:97-103,
 * src/IBCMatrixManipulations.cpp:84-106 and PlotPointsCPDiff :254-416): per point
 * xp[3i..3i+2] its 64 interpolation entries cols[64i..], vals[64i..] in the
 * operator's column layout, the stencil nodes that lie across an IBC from the
 * point moved to that IBC's DOF columns.  u(xp_i) = sum_e vals[64i+e] x[cols[64i+e]].
 * CPM_ERR_BASEPOINT_OUTSIDE_TUBE if a stencil leaves the tube; CPM_ERR_UNSUPPORTED if
 * an entry lies across two IBCs (it would need a 65th entry). */
int cpm_opset_plot_interp(cpm_opset_t op, int64_t n, const double *xp, int64_t *cols, double *vals);

/* The same evaluation rows as CSR (ptr: n + 1): each point's 64 entries, then one more
 * copy of every entry that lies across several IBCs for each further IBC, in that IBC's
 * DOF column (MoveToIBCColumns keeps one copy per IBC, src/IBCMatrixManipulations.cpp:189-216).
 * nnz query with ptr = NULL. */
int cpm_opset_plot_interp_csr(cpm_opset_t op, int64_t n, const double *xp, int64_t *nnz, int64_t *ptr, int64_t *cols,
                              double *vals);

/* The operator of the nearest-node baselines (PoissonWithIBCNearest,
 * problems/PoissonWithIBCNearest.cpp:73-89): the tube's plain L and E with
 * identity rows (Dirichlet values) at the n_rows given tube rows (device
 * indices). */
int cpm_opset_create_identity(cpm_tube_t t, int64_t n_rows, const int64_t *rows, cpm_opset_t *out);

int cpm_opset_destroy(cpm_opset_t op);

/* ---- Operator apply and solve --------------------------------------------
 * GeneralizedBiCGStabSystem::Multiply (src/GeneralizedBiCGStabSystem.h:191-233)
 * = Solver::Multiply (src/Solver.cpp:122-138):
 *   y = x on identity rows, else m x + n (L_qq x_q + sum_{c!=q} L_qc (E~x)_c).
 * x, y: host arrays of D*k doubles, RHS-major (x[j*D + r] is row r of RHS j). */
int cpm_apply(cpm_opset_t op, double m, double n, int32_t k, const double *x, double *y);

/* Explicit heat step (HeatWithIBC::TimeStep with time_stepping_method 0,
 * problems/HeatWithIBC.cpp:129-132): u_out = Efull (u + dt Lfull u), FP64, k
 * right-hand sides RHS-major; the caller sets the Dirichlet value rows after it. */
int cpm_explicit_step(cpm_opset_t op, double dt, int32_t k, const double *u, double *u_out);

/* Gray-Scott step of ReactionDiffusionWithIBC::TimeStep (problems/ReactionDiffusionWithIBC.cpp:93-117),
 * in place on host arrays of D doubles: u <- Efull (u + nu_u dt Lfull u + dt (-u v^2 + F (1 - u))),
 * v <- Efull (v + nu_v dt Lfull v + dt (u v^2 - (F + k) v)), the reaction terms from the old u, v,
 * nu_u = (dx / 3)^2, nu_v = nu_u / 3 (the reference uses F = 0.054, k = 0.063); the caller sets
 * the Dirichlet value rows afterwards. */
int cpm_gray_scott_step(cpm_opset_t op, double dt, double F, double k, double *u, double *v);
/* Same with device pointers: row-major [D][kslots] arrays (kslots 1 or 32),
 * FP64 or FP32 (fp32 = 1), t_dev a caller-owned scratch array of the same
 * shape for E~x.  Enqueued on the library stream, asynchronous (cpm_sync). */
int cpm_apply_device(cpm_opset_t op, double m, double n, int32_t kslots, int32_t fp32, const void *x_dev, void *t_dev,
                     void *y_dev);

/* Launch shapes of an operator's 32-slot E passes, as blocks per SM of their
 * grid-stride loops: the FP32 bulk pass, the IBC patch pass and the FP64 bulk
 * pass (0 keeps the built-in default).  They never change results.  No
 * counterpart in the reference, whose E is a CPU sparse product. */
typedef struct {
    int32_t e32_blocks_per_sm, patch_blocks_per_sm, e64_blocks_per_sm;
    float e32_us, patch_us, e64_us;                      /* the chosen shapes' mean launch times */
    float e32_default_us, patch_default_us, e64_default_us; /* the defaults' */
} cpm_tune_result;
/* Set the shapes by hand (0: default). */
int cpm_opset_set_launch(cpm_opset_t op, int32_t e32_blocks_per_sm, int32_t patch_blocks_per_sm, int32_t e64_blocks_per_sm);
/* The autotuner: time each pass over candidate shapes (reps launches each, on
 * scratch vectors it allocates and frees; the FP64 pass only when with_fp64)
 * on the calling thread's stream, keep the fastest with the operator (the
 * default unless another is at least 2 % faster) and report the times in
 * *out (may be NULL).  Blocks until done. */
int cpm_opset_autotune(cpm_opset_t op, int32_t reps, int32_t with_fp64, cpm_tune_result *out);

/* Allocation-free variant of cpm_apply_device.  It has no counterpart in the
 * reference; it exists for callers that cannot allocate device memory when
 * they apply the operator: applications whose device memory is entirely owned
 * by their own pool, and latency-critical loops in which a cudaMalloc or
 * cudaFree would synchronise the device and stall other streams.
 * Inputs and outputs are caller-owned as in cpm_apply_device; the E~x scratch
 * lives in one fixed device array of CPM_NOALLOC_SCRATCH_BYTES (32 MiB) that
 * every GPU which loads this library holds until the process exits.
 * D * kslots * (4 or 8 bytes) above that limit returns CPM_ERR_INVALID_ARG.
 * The first call on a device looks up the array's device address; make that
 * first call before any stream capture, with the library's device current.
 * The address is kept for the life of the process and stays valid only while
 * the device's primary context lives: after cudaDeviceReset (or anything else
 * that destroys the primary context) this entry point must not be called again
 * in the same process.
 * All calls share the one array, which keeps the previous call's contents
 * (every entry is rewritten before it is read, nothing needs clearing):
 * calls that overlap on the GPU race. */
#define CPM_NOALLOC_SCRATCH_BYTES (32u * 1024u * 1024u)
int cpm_apply_device_noalloc(cpm_opset_t op, double m, double n, int32_t kslots, int32_t fp32, const void *x_dev,
                             void *y_dev);

typedef struct cpm_solve_opts {
    double tol;             /* relative residual, reference 1e-10 (src/Solver.cpp:110) */
    int32_t max_iters;      /* reference 100000 */
    int32_t precision;      /* 0 plain FP64 BiCGStab, 1 FP32 BiCGStab refined in FP64 (reliable updates) */
    int32_t precond;        /* 0 identity, 1 diagonal, 2 jacobi (Defines.h:13-18) */
    int32_t precond_iters;  /* jacobi sweeps (Solver::SetPrecond, src/Solver.cpp:115-120) */
    double inner_tol;       /* precision 1: the FP32 residual reduction (0: 0.1) after which the
                               FP64 true residual replaces it (one refinement step) */
    int32_t max_refine;     /* FP64 refinement steps (default 400) */
    int32_t refine_every;   /* precision 1: iterations between reliable-update points, one of
                               1, 2, 4, 8, 16, 32 (0: 32) */
} cpm_solve_opts;

typedef struct cpm_solve_stats {
    int32_t iterations;      /* total BiCGStab iterations (inner iterations for precision 1) */
    int32_t refinements;     /* FP64 residual evaluations */
    int32_t restarts;
    int32_t status;          /* cpm_status of this right-hand side */
    double rel_residual;     /* final ||b - A x|| / ||b|| in FP64 */
    double seconds;          /* device time of the solve */
    int32_t fp64_fallback;   /* precision 1: 1 if the mixed solve did not converge and the plain
                                FP64 path solved this right-hand side again from x = 0 */
    int32_t pad;
} cpm_solve_stats;

/* Solver::Init(m, n, L, E, precond, identity_rows) (src/Solver.cpp:8-68):
 * binds (m, n) to an operator set and allocates k slot columns of solver state. */
int cpm_solver_create(cpm_opset_t op, double m, double n, int32_t kslots, cpm_solver_t *out);

/* Solver::Solve (src/Solver.cpp:69-114) for k right-hand sides at once (k <= kslots);
 * b, x: host, RHS-major D*k.  stats: k entries (may be NULL). */
int cpm_solve(cpm_solver_t s, int32_t k, const double *b, double *x, const cpm_solve_opts *opts, cpm_solve_stats *stats);
/* Device-resident variant: b_dev/x_dev are row-major [D][kslots] FP64 device arrays. */
int cpm_solve_device(cpm_solver_t s, int32_t k, const void *b_dev, void *x_dev, const cpm_solve_opts *opts,
                     cpm_solve_stats *stats);

int cpm_solver_destroy(cpm_solver_t s);

/* ---- Heat-method geodesic distance -----------------------------------------
 * GeodesicDistance::ComputeDistance(Tube&, IBCSubsets&, dt)
 * (problems/GeodesicDistance.cpp:11-69) from a point source (a Point IBC,
 * order 1, on_ibc_tolerance 0.1 dx^2): heat solve (m = 1, n = -dt), normalised
 * normal-projected gradient, divergence, Poisson solve (m = 0, n = 1),
 * phi -= min phi, repeated twice more on E phi.  create builds the IBC system
 * (D rows, returned in D_out).  run solves the heat step in FP64 with
 * `heat_sweeps` damped Jacobi sweeps per preconditioner call (<= 0: 2000, as
 * problems/GeodesicDistance.cpp:117-119), and the three Poisson steps with
 * `precision` 0 (plain FP64) or 1 (FP32 + FP64 reliable updates), all to
 * relative residual `tol`; it writes phi on the D rows (tube rows in device
 * order) and the 4 iteration counts. */
typedef struct cpm_geodesic_s *cpm_geodesic_t;
int cpm_geodesic_create(cpm_tube_t t, const double *source, cpm_geodesic_t *out, int64_t *D_out);
int cpm_geodesic_run(cpm_geodesic_t g, double dt, int32_t precision, double tol, int32_t heat_sweeps, double *phi_out,
                     int32_t *iters_out);
int cpm_geodesic_destroy(cpm_geodesic_t g);

/* Heat-method geodesic distance from up to 32 sources at once.  No counterpart
 * in the reference, whose GeodesicDistance::ComputeDistance serves one source per
 * call (problems/GeodesicDistance.cpp:11-69).  create builds one operator for all
 * of them: the tube's stencils with each source's point IBC (order 1,
 * on_ibc_tolerance 0.1 dx^2) applied to its own slot only; D_out = N + the
 * largest DOF count.  run performs cpm_geodesic_run's steps on every source at
 * once, in FP64 (the heat step with `heat_sweeps` damped Jacobi sweeps, <= 0:
 * 2000), and writes phi source-major: phi_out[k * D + r], the tube rows in
 * device order, then source k's own DOF rows (the rest of its rows are 0);
 * iters_out[4 k .. 4 k + 3] the heat and three Poisson iteration counts.  Each
 * source's phi equals its cpm_geodesic_run result up to rounding. */
typedef struct cpm_geodesic_batch_s *cpm_geodesic_batch_t;
int cpm_geodesic_batch_create(cpm_tube_t t, int32_t n_src, const double *sources, cpm_geodesic_batch_t *out,
                              int64_t *D_out);
int cpm_geodesic_batch_run(cpm_geodesic_batch_t g, double dt, double tol, int32_t heat_sweeps, double *phi_out,
                           int32_t *iters_out);
int cpm_geodesic_batch_destroy(cpm_geodesic_batch_t g);

/* GeodesicDistanceNearest::ComputeDistance(Tube&, ibc_idx, inside_ibc_idx,
 * inside_ibc_idx_dist, dt) (problems/GeodesicDistanceNearest.cpp:11-53): the
 * plain tube operator with identity rows at the constraint nodes `ibc_rows`
 * (every curve's list, concatenated in order; device row indices), and
 * smoothed heat sources SmoothH(-dist) at `inside_rows`.  The heat step
 * solves, as the reference does, the TRANSPOSE of I - dt (diag(L) + (L -
 * diag(L)) E) with the constraint rows set to identity rows; the reference
 * factorises it with a sparse LU (:103-133), run solves it in FP64 by
 * BiCGStab with `heat_sweeps` damped Jacobi sweeps per preconditioner call
 * (<= 0: 2000) to relative residual `tol`.  The three Poisson steps (m = 0,
 * n = 1, diagonal preconditioner) run in `precision` 0 or 1.  run writes phi on
 * the N tube rows (device order; the reference returns plotE * phi, which
 * cpm_opset_plot_interp of a plain operator set gives) and the 4 iteration
 * counts. */
typedef struct cpm_geodesic_nearest_s *cpm_geodesic_nearest_t;
int cpm_geodesic_nearest_create(cpm_tube_t t, int64_t n_ibc, const int64_t *ibc_rows, int64_t n_inside,
                                const int64_t *inside_rows, const double *inside_dist, cpm_geodesic_nearest_t *out);
int cpm_geodesic_nearest_run(cpm_geodesic_nearest_t g, double dt, int32_t precision, double tol, int32_t heat_sweeps,
                             double *phi_out, int32_t *iters_out);
int cpm_geodesic_nearest_destroy(cpm_geodesic_nearest_t g);

/* ---- Serving: continuous batching ------------------------------------------
 * No counterpart in the reference (its Solve is one blocking call per RHS,
 * src/Solver.cpp:104-113).  A server owns a 32-slot solver on one operator
 * (opset, m, n), mixed precision (opts->precision 1) or plain FP64 (0), with
 * the diagonal preconditioner.  submit queues a
 * right-hand side (D doubles, copied) with a caller tag; step admits queued
 * requests into free slots (each slot starts alone; the others keep their
 * state), runs one iteration graph if any slot is busy, and harvests finished
 * slots (a request the mixed path cannot converge is solved again by a 1-slot
 * plain FP64 solver at harvest, stats.fp64_fallback = 1); poll pops one finished request (returns 1, or 0 if none) with its
 * solution (D doubles, caller buffer or NULL), stats (stats.seconds = time
 * from admission into a slot to harvest) and latency (seconds from submit to
 * harvest, queueing included).  submit_device takes a device right-hand side
 * (D doubles, read when the request is admitted) and a device destination for
 * its solution (written when it finishes; poll then returns no x).
 * device_bytes estimates the device memory one 32-slot batch of a server on
 * `op` allocates, for admission by free HBM.  Solvers and servers run on
 * streams of their own, ordered after the work the calling thread queued on
 * the library stream; every call returns with its work complete. */
typedef struct cpm_server_s *cpm_server_t;
int cpm_server_create(cpm_opset_t op, double m, double n, const cpm_solve_opts *opts, cpm_server_t *out);
/* The same server over `batches` (1 to 8) 32-slot solvers, each on its own
 * stream: every step launches each busy batch's iteration graph before waiting
 * for any, so the batches' kernels overlap on the GPU (32 x batches slots). */
int cpm_server_create_batches(cpm_opset_t op, double m, double n, const cpm_solve_opts *opts, int32_t batches,
                              cpm_server_t *out);
int cpm_server_submit(cpm_server_t s, const double *b, int64_t tag);
int cpm_server_submit_device(cpm_server_t s, const void *b_dev, void *x_dev, int64_t tag);
int cpm_server_step(cpm_server_t s, int32_t *active, int32_t *queued, int32_t *finished);
/* step, pipelined: harvests what the previous call launched, then admits and
 * launches the next graphs and returns without waiting for them, so the caller's
 * polls (the host copies of the finished solutions) overlap them; a finished
 * request becomes visible one call later than with cpm_server_step.  A call that
 * leaves no slot busy and nothing queued waits for its own work.  Device
 * destinations are written in stream order before the calling thread's later
 * work on its stream. */
int cpm_server_step_async(cpm_server_t s, int32_t *active, int32_t *queued, int32_t *finished);
int cpm_server_poll(cpm_server_t s, int64_t *tag, double *x, cpm_solve_stats *stats, double *latency);
int cpm_server_destroy(cpm_server_t s);
int64_t cpm_server_device_bytes(cpm_opset_t op);

/* Synchronise the calling thread's stream (the library stream unless
 * cpm_set_thread_stream chose another). */
int cpm_sync(void);

/* The calling thread's CUDA stream (a cudaStream_t): the library stream unless
 * cpm_set_thread_stream chose another.  For callers that order their own work
 * or timing events with the library's. */
void *cpm_get_stream(void);

/* Queue the calling thread's library work (builds, applies, geodesics, the
 * entry ordering of solver calls) on `stream`, a cudaStream_t of the current
 * device that outlives its use here, instead of the library stream; NULL goes
 * back to the library stream.  Threads that each set a stream of their own
 * run their surfaces' work concurrently on the device.  No counterpart in the
 * reference, whose calls are blocking and single-threaded. */
int cpm_set_thread_stream(void *stream);

/* Number of kernels this library has launched in this process (graph
 * launches count their kernel nodes). */
int64_t cpm_launch_count(void);

#ifdef __cplusplus
}
#endif

#endif /* CPM_GPU_H */
