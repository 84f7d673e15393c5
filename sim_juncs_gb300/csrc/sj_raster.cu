// Device rasteriser (material classes per E-component Yee point) and the
// combo/bounding-box passes that turn class maps into the stepper's
// one-byte-per-voxel material index.
//
// The CSG evaluation restates composite_object::in and the primitives'
// in() (src/cgs.cpp:34-120, 403-449) with the reference's operation order:
// matrix rows are summed left to right starting from 0 (src/geometry.hpp:88-99),
// dot products left to right (src/geometry.hpp:199-201), and no fused
// multiply-add, so that points lying exactly on a face get the same answer.
#include "sj_internal.h"

namespace sj {

__device__ __forceinline__ void mat_vec(const double* __restrict__ m, double x, double y, double z,
                                        double& ox, double& oy, double& oz) {
    ox = __dadd_rn(__dadd_rn(__dadd_rn(0.0, __dmul_rn(m[0], x)), __dmul_rn(m[1], y)), __dmul_rn(m[2], z));
    oy = __dadd_rn(__dadd_rn(__dadd_rn(0.0, __dmul_rn(m[3], x)), __dmul_rn(m[4], y)), __dmul_rn(m[5], z));
    oz = __dadd_rn(__dadd_rn(__dadd_rn(0.0, __dmul_rn(m[6], x)), __dmul_rn(m[7], y)), __dmul_rn(m[8], z));
}

// Evaluate one region's postfix program at r; returns in_root(r) in {0,1}.
// The operand stack is a 64-bit word: push = shift left, pop = shift right.
__device__ int eval_program(const sj_csg_node* __restrict__ nodes, int n, double x, double y,
                            double z) {
    unsigned long long stk = 0;
    for (int q = 0; q < n; ++q) {
        const sj_csg_node& nd = nodes[q];
        const int op = nd.op;
        int v = 0;
        if (op <= SJ_CSG_PLANE) {
            double rx, ry, rz;
            mat_vec(nd.m, x, y, z, rx, ry, rz);
            if (op == SJ_CSG_PLANE) {
                const double d = __dadd_rn(__dadd_rn(__dmul_rn(rx, nd.p[0]), __dmul_rn(ry, nd.p[1])),
                                           __dmul_rn(rz, nd.p[2]));
                v = d > nd.p[3] ? 0 : 1;
            } else {
                double qx, qy, qz;
                mat_vec(nd.t, __dsub_rn(rx, nd.c[0]), __dsub_rn(ry, nd.c[1]), __dsub_rn(rz, nd.c[2]),
                        qx, qy, qz);
                bool out;
                if (op == SJ_CSG_BOX) {
                    out = fabs(qx) > nd.p[0] || fabs(qy) > nd.p[1] || fabs(qz) > nd.p[2];
                } else if (op == SJ_CSG_SPHERE) {
                    const double s2 = __dadd_rn(__dadd_rn(__dadd_rn(0.0, __dmul_rn(qx, qx)), __dmul_rn(qy, qy)),
                                                __dmul_rn(qz, qz));
                    out = __dsqrt_rn(s2) > nd.p[0];
                } else {  // cylinder: p = height, r1^2, r2^2
                    const double h = nd.p[0], r1 = nd.p[1], r2 = nd.p[2];
                    if (qz < 0 || qz > h) {
                        out = true;
                    } else {
                        const double cr = __dadd_rn(__dmul_rn(qx, qx), __dmul_rn(qy, qy));
                        out = __dmul_rn(cr, h) > __dadd_rn(__dmul_rn(__dsub_rn(r2, r1), qz), __dmul_rn(r1, h));
                    }
                }
                v = out ? nd.invert : 1 - nd.invert;
            }
            stk = (stk << 1) | (unsigned long long)v;
        } else if (op == SJ_CSG_UNION || op == SJ_CSG_INTERSECT) {
            const int b = (int)(stk & 1ull);
            stk >>= 1;
            const int a = (int)(stk & 1ull);
            stk >>= 1;
            v = nd.invert ^ (op == SJ_CSG_UNION ? (a | b) : (a & b));
            stk = (stk << 1) | (unsigned long long)v;
        } else if (op == SJ_CSG_PASS) {
            const int a = (int)(stk & 1ull);
            stk = (stk & ~1ull) | (unsigned long long)(nd.invert ^ a);
        } else if (op == SJ_CSG_CONST) {
            stk = (stk << 1) | (unsigned long long)(nd.invert & 1);
        } else {  // NOOP
            stk = (stk << 1);
        }
    }
    return (int)(stk & 1ull);
}

// Region start table carried by value in the kernel's parameters.
struct RegionStarts {
    int s[SJ_MAX_REGIONS + 1];
    __device__ int operator[](int g) const { return s[g]; }
};

// One thread per voxel: masks for the Ex, Ey and Ez points.  Starts is a
// device pointer to the region start table or a RegionStarts value.
template <typename Starts>
__global__ void k_rasterize(const sj_csg_node* __restrict__ nodes, const Starts rstart,
                            int n_regions, int nx, int ny, int nz, double dx, double ox, double oy,
                            double oz, uint8_t* __restrict__ masks, long long cpitch, int px) {
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    const long long total = (long long)nx * ny * nz;
    if (t >= total) return;
    const int i = (int)(t % nx);
    const long long r = t / nx;
    const int j = (int)(r % ny);
    const int k = (int)(r / ny);
    const long long o = ((long long)k * ny + j) * px + i;
    for (int c = 0; c < 3; ++c) {
        const double x = __dadd_rn(ox, __dmul_rn((double)i + (c == 0 ? 0.5 : 0.0), dx));
        const double y = __dadd_rn(oy, __dmul_rn((double)j + (c == 1 ? 0.5 : 0.0), dx));
        const double z = __dadd_rn(oz, __dmul_rn((double)k + (c == 2 ? 0.5 : 0.0), dx));
        unsigned m = 0;
        for (int g = 0; g < n_regions; ++g) {
            const int s = rstart[g], e = rstart[g + 1];
            if (eval_program(nodes + s, e - s, x, y, z)) m |= 1u << g;
        }
        masks[c * cpitch + o] = (uint8_t)m;
    }
}

cudaError_t launch_rasterize(const sj_csg_node* d_nodes, const int* d_region_start, int n_regions,
                             int nx, int ny, int nz, double dx, const double* origin,
                             uint8_t* d_masks, long long mask_pitch_elems, int px, cudaStream_t s) {
    const long long total = (long long)nx * ny * nz;
    const unsigned blocks = (unsigned)((total + 255) / 256);
    k_rasterize<const int*><<<blocks, 256, 0, s>>>(d_nodes, d_region_start, n_regions, nx, ny, nz, dx,
                                                   origin[0], origin[1], origin[2], d_masks, mask_pitch_elems,
                                                   px);
    return cudaGetLastError();
}

// ------------------------------------------------------------ smoothing
// Stochastic smoothing (cgs_material_function::in_bound, src/disp.cpp:264-283):
// at each E-component Yee point, region g's count is in(r) plus in(r + d_j)
// over the n_offs offsets, r + d_j formed by one rounded add per axis as there.
// A point's key packs the counts 8 bits per region (at most 8 * 31 + 1 = 249,
// so the all-ones word never occurs and marks an empty slot of the key set).
constexpr unsigned long long SMOOTH_EMPTY = ~0ull;

__device__ __forceinline__ unsigned smooth_slot(unsigned long long key, unsigned cap) {
    key ^= key >> 29;
    key *= 0xbf58476d1ce4e5b9ull;
    key ^= key >> 32;
    return (unsigned)key & (cap - 1);
}

// Insert key into the open-addressing set (cap a power of two); at most cap
// probes, after which *overflow is raised.
__device__ void smooth_insert(unsigned long long* set, unsigned cap, unsigned long long key, int* overflow) {
    unsigned h = smooth_slot(key, cap);
    for (unsigned probe = 0; probe < cap; ++probe) {
        const unsigned long long cur = ((volatile unsigned long long*)set)[h];
        if (cur == key) return;
        if (cur == SMOOTH_EMPTY) {
            const unsigned long long prev = atomicCAS(set + h, SMOOTH_EMPTY, key);
            if (prev == SMOOTH_EMPTY || prev == key) return;
        }
        h = (h + 1) & (cap - 1);
    }
    atomicExch(overflow, 1);
}

// One thread per voxel: keys of the Ex, Ey and Ez points; with a set, every
// distinct key also goes into it (one insert per distinct key of a warp).
__global__ void k_rasterize_counts(const sj_csg_node* __restrict__ nodes, const int* __restrict__ rstart,
                                   int n_regions, int nx, int ny, int nz, double dx, double ox, double oy,
                                   double oz, const double* __restrict__ offs, int n_offs,
                                   unsigned long long* __restrict__ keys, long long kpitch, int px,
                                   unsigned long long* __restrict__ set, unsigned cap, int* __restrict__ overflow) {
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    const long long total = (long long)nx * ny * nz;
    if (t >= total) return;
    const int i = (int)(t % nx);
    const long long r = t / nx;
    const int j = (int)(r % ny);
    const int k = (int)(r / ny);
    const long long o = ((long long)k * ny + j) * px + i;
    for (int c = 0; c < 3; ++c) {
        const double x = __dadd_rn(ox, __dmul_rn((double)i + (c == 0 ? 0.5 : 0.0), dx));
        const double y = __dadd_rn(oy, __dmul_rn((double)j + (c == 1 ? 0.5 : 0.0), dx));
        const double z = __dadd_rn(oz, __dmul_rn((double)k + (c == 2 ? 0.5 : 0.0), dx));
        unsigned long long key = 0;
        for (int g = 0; g < n_regions; ++g) {
            const int s = rstart[g], e = rstart[g + 1];
            unsigned cnt = (unsigned)eval_program(nodes + s, e - s, x, y, z);
            for (int q = 0; q < n_offs; ++q)
                cnt += (unsigned)eval_program(nodes + s, e - s, __dadd_rn(x, offs[3 * q]),
                                              __dadd_rn(y, offs[3 * q + 1]), __dadd_rn(z, offs[3 * q + 2]));
            key |= (unsigned long long)cnt << (8 * g);
        }
        keys[c * kpitch + o] = key;
        if (set) {
            const unsigned peers = __match_any_sync(__activemask(), key);
            if ((threadIdx.x & 31) == (unsigned)(__ffs(peers) - 1)) smooth_insert(set, cap, key, overflow);
        }
    }
}

cudaError_t launch_rasterize_counts(const sj_csg_node* d_nodes, const int* d_region_start, int n_regions,
                                    int nx, int ny, int nz, double dx, const double* origin,
                                    const double* d_offs, int n_offs, unsigned long long* d_keys,
                                    long long key_pitch_elems, int px, unsigned long long* d_set,
                                    unsigned cap, int* d_overflow, cudaStream_t s) {
    const long long total = (long long)nx * ny * nz;
    const unsigned blocks = (unsigned)((total + 255) / 256);
    k_rasterize_counts<<<blocks, 256, 0, s>>>(d_nodes, d_region_start, n_regions, nx, ny, nz, dx, origin[0],
                                              origin[1], origin[2], d_offs, n_offs, d_keys, key_pitch_elems,
                                              px, d_set, cap, d_overflow);
    return cudaGetLastError();
}

// Replace each point's key by its index in the sorted list of distinct keys
// (n_keys <= 256): the point's material class.
__global__ void k_class_assign(const unsigned long long* __restrict__ keys, long long pitch, int nx, int ny,
                               int nz, int px, const unsigned long long* __restrict__ sorted, int n_keys,
                               uint8_t* __restrict__ cls) {
    __shared__ unsigned long long sk[256];
    for (int q = threadIdx.x; q < n_keys; q += blockDim.x) sk[q] = sorted[q];
    __syncthreads();
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    const long long total = (long long)nx * ny * nz;
    if (t >= total) return;
    const int i = (int)(t % nx);
    const long long r = t / nx;
    const int j = (int)(r % ny);
    const int k = (int)(r / ny);
    const long long o = ((long long)k * ny + j) * px + i;
    for (int c = 0; c < 3; ++c) {
        const unsigned long long key = keys[c * pitch + o];
        int lo = 0, hi = n_keys - 1;
        while (lo < hi) {
            const int mid = (lo + hi) >> 1;
            if (sk[mid] < key)
                lo = mid + 1;
            else
                hi = mid;
        }
        cls[c * pitch + o] = (uint8_t)lo;
    }
}

cudaError_t launch_class_assign(const unsigned long long* d_keys, long long pitch, int nx, int ny, int nz,
                                int px, const unsigned long long* d_sorted, int n_keys, uint8_t* d_cls,
                                cudaStream_t s) {
    const long long total = (long long)nx * ny * nz;
    k_class_assign<<<(unsigned)((total + 255) / 256), 256, 0, s>>>(d_keys, pitch, nx, ny, nz, px, d_sorted,
                                                                   n_keys, d_cls);
    return cudaGetLastError();
}

// Mark every (class_x, class_y, class_z) triple present in a 2^24-bit set.
__global__ void k_combo_mark(const uint8_t* __restrict__ cls, long long cpitch, int nx, int ny,
                             int nz, int px, uint32_t* __restrict__ bitmap) {
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    const long long total = (long long)nx * ny * nz;
    if (t >= total) return;
    const int i = (int)(t % nx);
    const long long r = t / nx;
    const int j = (int)(r % ny);
    const int k = (int)(r / ny);
    const long long o = ((long long)k * ny + j) * px + i;
    const uint32_t key = (uint32_t)cls[o] | ((uint32_t)cls[cpitch + o] << 8) |
                         ((uint32_t)cls[2 * cpitch + o] << 16);
    const uint32_t bit = 1u << (key & 31u);
    uint32_t* w = bitmap + (key >> 5);
    if ((*((volatile uint32_t*)w) & bit) == 0) atomicOr(w, bit);
}

cudaError_t launch_combo_mark(const uint8_t* d_cls, long long cpitch, int nx, int ny, int nz,
                              int px, uint32_t* d_bitmap, cudaStream_t s) {
    const long long total = (long long)nx * ny * nz;
    k_combo_mark<<<(unsigned)((total + 255) / 256), 256, 0, s>>>(d_cls, cpitch, nx, ny, nz, px, d_bitmap);
    return cudaGetLastError();
}

// The set bits of the triple bitmap as a key list (unordered; the host sorts
// the at most cap it reads back).  *count gets the number of set bits.
__global__ void k_combo_compact(const uint32_t* __restrict__ bitmap, int n_words, uint32_t* __restrict__ keys,
                                int cap, int* __restrict__ count) {
    for (int w = blockIdx.x * blockDim.x + threadIdx.x; w < n_words; w += gridDim.x * blockDim.x) {
        uint32_t bits = bitmap[w];
        while (bits) {
            const int b = __ffs(bits) - 1;
            bits &= bits - 1;
            const int slot = atomicAdd(count, 1);
            if (slot < cap) keys[slot] = (uint32_t)w * 32u + (uint32_t)b;
        }
    }
}

cudaError_t launch_combo_compact(const uint32_t* d_bitmap, int n_words, uint32_t* d_keys, int cap, int* d_count,
                                 cudaStream_t s) {
    k_combo_compact<<<608, 256, 0, s>>>(d_bitmap, n_words, d_keys, cap, d_count);
    return cudaGetLastError();
}

// Replace each voxel's triple by its index in the sorted key list.
__global__ void k_combo_assign(const uint8_t* __restrict__ cls, long long cpitch, int nx, int ny,
                               int nz, int px, const uint32_t* __restrict__ keys, int n_keys,
                               uint8_t* __restrict__ combo) {
    __shared__ uint32_t sk[256];
    for (int q = threadIdx.x; q < n_keys; q += blockDim.x) sk[q] = keys[q];
    __syncthreads();
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    const long long total = (long long)nx * ny * nz;
    if (t >= total) return;
    const int i = (int)(t % nx);
    const long long r = t / nx;
    const int j = (int)(r % ny);
    const int k = (int)(r / ny);
    const long long o = ((long long)k * ny + j) * px + i;
    const uint32_t key = (uint32_t)cls[o] | ((uint32_t)cls[cpitch + o] << 8) |
                         ((uint32_t)cls[2 * cpitch + o] << 16);
    int lo = 0, hi = n_keys - 1;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (sk[mid] < key)
            lo = mid + 1;
        else
            hi = mid;
    }
    combo[o] = (uint8_t)lo;
}

cudaError_t launch_combo_assign(const uint8_t* d_cls, long long cpitch, int nx, int ny, int nz,
                                int px, const uint32_t* d_keys, int n_keys, uint8_t* d_combo,
                                cudaStream_t s) {
    const long long total = (long long)nx * ny * nz;
    k_combo_assign<<<(unsigned)((total + 255) / 256), 256, 0, s>>>(d_cls, cpitch, nx, ny, nz, px,
                                                                   d_keys, n_keys, d_combo);
    return cudaGetLastError();
}

// Bounding box of voxels whose combo carries a polarisation: box = {min i,j,k, max i,j,k}.
__global__ void k_disp_bbox(const uint8_t* __restrict__ combo, const uint8_t* __restrict__ cflag,
                            int nx, int ny, int nz, int px, int* box) {
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    const long long total = (long long)nx * ny * nz;
    if (t >= total) return;
    const int i = (int)(t % nx);
    const long long r = t / nx;
    const int j = (int)(r % ny);
    const int k = (int)(r / ny);
    const long long o = ((long long)k * ny + j) * px + i;
    if (cflag[combo[o]] & 1) {
        atomicMin(box + 0, i);
        atomicMin(box + 1, j);
        atomicMin(box + 2, k);
        atomicMax(box + 3, i);
        atomicMax(box + 4, j);
        atomicMax(box + 5, k);
    }
}

cudaError_t launch_disp_bbox(const uint8_t* d_combo, const uint8_t* d_cflag, int nx, int ny,
                             int nz, int px, int* d_box, cudaStream_t s) {
    const long long total = (long long)nx * ny * nz;
    k_disp_bbox<<<(unsigned)((total + 255) / 256), 256, 0, s>>>(d_combo, d_cflag, nx, ny, nz, px, d_box);
    return cudaGetLastError();
}

}  // namespace sj

namespace sj {
// 256-bin histogram of the combo map (voxel counts per material combo).
__global__ void k_combo_hist(const uint8_t* __restrict__ combo, int nx, int ny, int nz, int px,
                             unsigned long long* __restrict__ hist) {
    __shared__ unsigned int h[256];
    for (int q = threadIdx.x; q < 256; q += blockDim.x) h[q] = 0;
    __syncthreads();
    const long long total = (long long)nx * ny * nz;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
         t += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(t % nx);
        const long long r = t / nx;
        const int j = (int)(r % ny);
        const int k = (int)(r / ny);
        atomicAdd(&h[combo[((long long)k * ny + j) * px + i]], 1u);
    }
    __syncthreads();
    for (int q = threadIdx.x; q < 256; q += blockDim.x)
        if (h[q]) atomicAdd(hist + q, (unsigned long long)h[q]);
}

cudaError_t launch_combo_hist(const uint8_t* d_combo, int nx, int ny, int nz, int px,
                              unsigned long long* d_hist, cudaStream_t s) {
    k_combo_hist<<<608, 256, 0, s>>>(d_combo, nx, ny, nz, px, d_hist);
    return cudaGetLastError();
}
}  // namespace sj

// ---------------------------------------------------------------------------
// Allocation-free rasteriser (sj_rasterize_static).
//
// The concatenated CSG programs live in one file-scope device array instead
// of cudaMalloc'd buffers; the region start table travels by value in the
// kernel's parameters.  Host code never names the array directly: its device
// address comes from cudaGetSymbolAddress, looked up with the device current
// and cached per device together with the context it was taken in, so a
// context torn down and created again (cudaDeviceReset) gets a fresh lookup.
#include <cuda.h>
#include <mutex>

namespace sj {

constexpr size_t RASTER_SCRATCH_BYTES = (size_t)SJ_RASTER_STATIC_NODES * sizeof(sj_csg_node);

static __device__ __align__(256) unsigned char g_raster_scratch[RASTER_SCRATCH_BYTES];

namespace {
constexpr int MAX_DEVICES = 64;
std::mutex g_scratch_mu;
unsigned char* g_scratch_ptr[MAX_DEVICES] = {};
CUcontext g_scratch_ctx[MAX_DEVICES] = {};

typedef CUresult (*CtxGetCurrentFn)(CUcontext*);

// The driver's current context, through the runtime's entry-point table (the
// library links only the CUDA runtime).
cudaError_t current_context(CUcontext* out) {
    static CtxGetCurrentFn fn = nullptr;
    if (!fn) {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        cudaError_t e = cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 4000, cudaEnableDefault, &q);
        if (e != cudaSuccess) return e;
        if (q != cudaDriverEntryPointSuccess || !p) return cudaErrorNotSupported;
        fn = reinterpret_cast<CtxGetCurrentFn>(p);
    }
    return fn(out) == CUDA_SUCCESS ? cudaSuccess : cudaErrorContextIsDestroyed;
}

// Device address of g_raster_scratch on the current device.
cudaError_t raster_scratch(unsigned char** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= MAX_DEVICES) return cudaErrorInvalidDevice;
    CUcontext ctx = nullptr;
    e = current_context(&ctx);
    if (e != cudaSuccess) return e;
    std::lock_guard<std::mutex> lock(g_scratch_mu);
    if (!ctx || !g_scratch_ptr[dev] || g_scratch_ctx[dev] != ctx) {
        // no context yet (first CUDA call of this thread) or a new one: the
        // lookup makes the device's primary context current if none is
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_raster_scratch);
        if (e != cudaSuccess) return e;
        e = current_context(&ctx);
        if (e != cudaSuccess) return e;
        g_scratch_ptr[dev] = static_cast<unsigned char*>(p);
        g_scratch_ctx[dev] = ctx;
    }
    *out = g_scratch_ptr[dev];
    return cudaSuccess;
}
}  // namespace

// Returns 0 or an SJ_E_* code; *msg gets a static description on failure.
int rasterize_static(const sj_grid_desc* g, const sj_scene_desc* sc, uint8_t* d_out, cudaStream_t s,
                     const char** msg) {
    if (!g || !sc || !d_out) {
        *msg = "NULL argument";
        return SJ_E_INVALID;
    }
    if (g->nx < 1 || g->ny < 1 || g->nz < 1 || !(g->dx > 0)) {
        *msg = "bad grid";
        return SJ_E_INVALID;
    }
    if (sc->n_regions < 0 || sc->n_regions > SJ_MAX_REGIONS || (sc->n_regions > 0 && !sc->regions)) {
        *msg = "scene n_regions must be in [0, 8]";
        return SJ_E_INVALID;
    }
    if (sc->smooth_n != 0) {
        *msg = "a smoothed scene has fill counts, not region masks (sj_rasterize_counts)";
        return SJ_E_INVALID;
    }
    RegionStarts start = {};
    for (int r = 0; r < sc->n_regions; ++r) {
        const sj_region_desc& rg = sc->regions[r];
        if (rg.n_nodes < 1 || !rg.nodes) {
            *msg = "region without CSG nodes";
            return SJ_E_INVALID;
        }
        int depth = 0;
        for (int q = 0; q < rg.n_nodes; ++q) {
            const int op = rg.nodes[q].op;
            if (op < 0 || op > SJ_CSG_NOOP) {
                *msg = "unknown CSG op";
                return SJ_E_INVALID;
            }
            if (op <= SJ_CSG_PLANE || op == SJ_CSG_CONST || op == SJ_CSG_NOOP)
                ++depth;
            else if (op == SJ_CSG_UNION || op == SJ_CSG_INTERSECT)
                depth = depth >= 2 ? depth - 1 : -1000;
            else if (depth < 1)
                depth = -1000;
            if (depth < 0 || depth > 64) {
                *msg = "malformed CSG program";
                return SJ_E_INVALID;
            }
        }
        if (depth != 1) {
            *msg = "CSG program must leave exactly one value";
            return SJ_E_INVALID;
        }
        if (start.s[r] + rg.n_nodes > SJ_RASTER_STATIC_NODES) {
            *msg = "scene has more CSG nodes than SJ_RASTER_STATIC_NODES (512)";
            return SJ_E_RANGE;
        }
        start.s[r + 1] = start.s[r] + rg.n_nodes;
    }
    unsigned char* base = nullptr;
    cudaError_t e = raster_scratch(&base);
    if (e != cudaSuccess) {
        *msg = "cudaGetSymbolAddress of the rasteriser scratch array failed";
        return SJ_E_CUDA;
    }
    // the program is overwritten in full by every call; nothing needs clearing
    sj_csg_node* d_nodes = reinterpret_cast<sj_csg_node*>(base);
    for (int r = 0; r < sc->n_regions && e == cudaSuccess; ++r)
        e = cudaMemcpyAsync(d_nodes + start.s[r], sc->regions[r].nodes,
                            (size_t)sc->regions[r].n_nodes * sizeof(sj_csg_node), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) {
        const long long nv = (long long)g->nx * g->ny * g->nz;
        const long long total = nv;
        const unsigned blocks = (unsigned)((total + 255) / 256);
        k_rasterize<RegionStarts><<<blocks, 256, 0, s>>>(d_nodes, start, sc->n_regions, g->nx, g->ny, g->nz,
                                                         g->dx, g->origin[0], g->origin[1], g->origin[2], d_out,
                                                         nv, g->nx);
        e = cudaGetLastError();
    }
    if (e != cudaSuccess) {
        *msg = "CUDA call failed in sj_rasterize_static";
        return SJ_E_CUDA;
    }
    return SJ_OK;
}

}  // namespace sj
