// Internal structures of the GB300 closest-point solve library.
//
// Layout in HBM (one GPU):
//   * Tube nodes are stored compactly, ordered by the Morton code of their 4^3
//     brick and, inside a brick, by the local slot l = (i&3)<<4 | (j&3)<<2 | (k&3).
//   * A dense brick map (NB^3 int32, NB = ceil(N1d/4)) gives the occupied-brick
//     rank; per rank a 64-bit occupancy mask and the index of its first node.
//     node(i,j,k) = start[rank] + popc(mask & ((1<<l)-1)) — no per-node
//     neighbour or stencil index tables are stored.
//   * Grid triplets are packed in 32 bits (10 bits per axis, N1d <= 1024).
//   * Operator rows: tube rows [0, N) in node order, then IBC DOF rows and
//     Dirichlet value rows [N, D) in the reference's column layout.
//   * Vectors of a k-slot batch are row-major [D][k] so one stencil gather
//     reads k contiguous values.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

#include <string>
#include <vector>

#include "../../include/cpm_gpu.h"

namespace cpm {

// ---------------------------------------------------------------- errors
void set_error(const std::string &msg);
int fail(int code, const std::string &msg);

#define CPM_CUDA_TRY(expr)                                                                       \
    do {                                                                                         \
        cudaError_t _e = (expr);                                                                 \
        if (_e != cudaSuccess)                                                                   \
            return ::cpm::fail(_e == cudaErrorMemoryAllocation ? CPM_ERR_OOM : CPM_ERR_CUDA,     \
                               std::string(#expr) + ": " + cudaGetErrorString(_e));              \
    } while (0)

#define CPM_TRY(expr)            \
    do {                         \
        int _rc = (expr);        \
        if (_rc != 0) return _rc; \
    } while (0)

// the stream the library's work is ordered on: the calling thread's current
// StreamScope stream, else the library stream
cudaStream_t stream();
cudaStream_t library_stream();
// while alive, stream() of this thread is s (a solver's own stream)
struct StreamScope {
    explicit StreamScope(cudaStream_t s);
    ~StreamScope();
    StreamScope(const StreamScope &) = delete;
    StreamScope &operator=(const StreamScope &) = delete;
    cudaStream_t prev;
};
// adds to the process-wide count of launched kernels (cpm_launch_count)
void count_launches(long long n);

// ---------------------------------------------------------------- device buffers
template <class T>
struct DBuf {
    T *p = nullptr;
    size_t n = 0;
    DBuf() = default;
    DBuf(const DBuf &) = delete;
    DBuf &operator=(const DBuf &) = delete;
    ~DBuf() { release(); }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
    }
    int alloc(size_t count) {
        release();
        if (count == 0) count = 1;
        cudaError_t e = cudaMalloc((void **)&p, count * sizeof(T));
        if (e != cudaSuccess) {
            p = nullptr;
            return fail(CPM_ERR_OOM, std::string("cudaMalloc: ") + cudaGetErrorString(e));
        }
        n = count;
        return 0;
    }
    int zero() {
        CPM_CUDA_TRY(cudaMemsetAsync(p, 0, n * sizeof(T), stream()));
        return 0;
    }
    int upload(const T *h, size_t count) {
        CPM_TRY(alloc(count));
        CPM_CUDA_TRY(cudaMemcpyAsync(p, h, count * sizeof(T), cudaMemcpyHostToDevice, stream()));
        return 0;
    }
    int upload(const std::vector<T> &h) { return upload(h.data(), h.size()); }
    int download(std::vector<T> &h, size_t count) const {
        h.resize(count);
        if (count) CPM_CUDA_TRY(cudaMemcpyAsync(h.data(), p, count * sizeof(T), cudaMemcpyDeviceToHost, stream()));
        CPM_CUDA_TRY(cudaStreamSynchronize(stream()));
        return 0;
    }
};

// Host array in page-locked memory.  A device-to-host cudaMemcpyAsync into
// pageable memory returns only once the copy (and so all earlier work on its
// stream) is done; into a PinnedArray it is queued like any other stream work.
template <class T>
struct PinnedArray {
    T *p = nullptr;
    size_t n = 0;
    PinnedArray() = default;
    PinnedArray(const PinnedArray &) = delete;
    PinnedArray &operator=(const PinnedArray &) = delete;
    ~PinnedArray() {
        if (p) cudaFreeHost(p);
    }
    int alloc(size_t count) {
        if (p) cudaFreeHost(p);
        p = nullptr;
        n = 0;
        cudaError_t e = cudaMallocHost((void **)&p, (count ? count : 1) * sizeof(T));
        if (e != cudaSuccess) {
            p = nullptr;
            return fail(CPM_ERR_OOM, std::string("cudaMallocHost: ") + cudaGetErrorString(e));
        }
        n = count;
        memset(p, 0, (count ? count : 1) * sizeof(T));
        return 0;
    }
    T *data() { return p; }
    const T *data() const { return p; }
    T &operator[](size_t i) { return p[i]; }
    const T &operator[](size_t i) const { return p[i]; }
};

// ---------------------------------------------------------------- geometry
struct SurfaceParams {
    int kind;
    double p[8];
    // mesh (triangles / segments) with a uniform cell grid for candidate search
    const double *verts;     // device, 3*nv
    const int32_t *prims;    // device, 3*np or 2*np
    int64_t nprims;
    const int32_t *cell_start;  // device, ncell+1
    const int32_t *cell_items;  // device
    double glo[3];
    double gh;
    int gn[3];
};

struct GridParams {
    double dx, xstart, radius;
    int N1d, NB;
};

__host__ __device__ inline uint32_t pack3(int i, int j, int k) { return ((uint32_t)i << 20) | ((uint32_t)j << 10) | (uint32_t)k; }
__host__ __device__ inline int unpack_i(uint32_t v) { return (int)(v >> 20); }
__host__ __device__ inline int unpack_j(uint32_t v) { return (int)((v >> 10) & 1023u); }
__host__ __device__ inline int unpack_k(uint32_t v) { return (int)(v & 1023u); }

// read-only view of the brick tables
struct BrickView {
    const int32_t *bmap;    // NB^3 -> rank or -1
    const uint64_t *bmask;  // per rank
    const int32_t *bstart;  // per rank
    int NB, N1d;
};

__device__ __forceinline__ int node_at(const BrickView &b, int i, int j, int k) {
    if (i < 0 || j < 0 || k < 0 || i >= b.N1d || j >= b.N1d || k >= b.N1d) return -1;
    int r = __ldg(&b.bmap[((size_t)(i >> 2) * b.NB + (j >> 2)) * b.NB + (k >> 2)]);
    if (r < 0) return -1;
    uint64_t m = __ldg(&b.bmask[r]);
    int l = ((i & 3) << 4) | ((j & 3) << 2) | (k & 3);
    if (!((m >> l) & 1ull)) return -1;
    return __ldg(&b.bstart[r]) + __popcll(m & ((1ull << l) - 1ull));
}

// ---------------------------------------------------------------- tube object
struct Mesh {
    DBuf<double> verts;
    DBuf<int32_t> prims, cell_start, cell_items;
    int64_t nprims = 0;
    double glo[3] = {0, 0, 0}, gh = 0;
    int gn[3] = {0, 0, 0};
};

struct SurfaceObj {
    cpm_surface_desc desc;  // host copy (mesh pointers not retained)
    Mesh mesh;
    SurfaceParams params() const;
};
// cell_h > 0: cell size of the mesh search grid (the tube radius); 0: automatic
int surface_init(SurfaceObj &s, const cpm_surface_desc *d, double cell_h);

}  // namespace cpm

struct cpm_tube_s {
    cpm::SurfaceObj surf;
    cpm::GridParams g;
    int p = 3;
    int64_t N = 0, nbricks = 0, nvisited = 0;
    cpm::DBuf<int32_t> bmap, bstart;
    cpm::DBuf<uint64_t> bmask;
    cpm::DBuf<uint32_t> key;    // packed triplet per node
    cpm::DBuf<double> cp, dist;  // 3N, N
    cpm::DBuf<uint32_t> base;   // packed base triplet per node
    cpm::DBuf<double> w;        // 12 per node: [d][j]
    int seed[3] = {0, 0, 0};    // grid triplet of the build's seed node
    cpm::BrickView view() const { return cpm::BrickView{bmap.p, bmask.p, bstart.p, g.NB, g.N1d}; }
};

namespace cpm {
// closest points of n device points (used by the opset build for cp-bar and IBC distances)
// max_dist bounds mesh searches (dist > max_dist is reported for farther points)
int closest_points_dev(const SurfaceParams &sp, int64_t n, const double *x, double *cp, double *dist, double max_dist);
// base points + weights of n device query points against a tube; err flag set on failure
int interp_weights_dev(const cpm_tube_s *t, int64_t n, const double *xq, uint32_t *base, double *w, int32_t *err);
}  // namespace cpm
