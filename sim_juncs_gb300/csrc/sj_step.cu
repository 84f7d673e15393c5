// Stepping kernels: probes (monitors + running DFT), the split H/E schedule,
// and small utilities.  The fused single-pass schedule lives in sj_fused.cu.
#include "sj_physics.cuh"

namespace sj {

constexpr int MAXF = 256;  // DFT frequencies per instance

__device__ __forceinline__ int find_inst(const long long* __restrict__ blk0, int n, long long b) {
    int lo = 0, hi = n - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (blk0[mid] <= b)
            lo = mid;
        else
            hi = mid - 1;
    }
    return lo;
}

// Copy an instance descriptor into shared memory (block-wide, ends with a sync).
template <typename real>
__device__ __forceinline__ void load_inst(const InstDev<real>* src, InstDev<real>* dst) {
    const int* s = reinterpret_cast<const int*>(src);
    int* d = reinterpret_cast<int*>(dst);
    const int nw = (int)(sizeof(InstDev<real>) / sizeof(int));
    for (int w = threadIdx.y * blockDim.x + threadIdx.x; w < nw; w += blockDim.x * blockDim.y) d[w] = s[w];
    __syncthreads();
}

// Last block of the grid advances the device step counter.  Every block of
// a launch reads `step` before any block can reach this point, so the
// increment never races with a reader of the same launch.
__device__ __forceinline__ void finish_block(DevState* st) {
    __syncthreads();
    if (threadIdx.x == 0 && threadIdx.y == 0 && threadIdx.z == 0) {
        __threadfence();
        const unsigned total = gridDim.x * gridDim.y * gridDim.z;
        const unsigned prev = atomicAdd(&st->done, 1u);
        if (prev == total - 1) {
            st->step += 1;
            st->done = 0;
            __threadfence();
        }
    }
}

// --------------------------------------------------------------- probes
// Monitor samples (src/disp.cpp:721-731: get_field every save_span steps,
// before the step) and the running DFT sums, read from the buffers that
// hold E^n and H^{n-1/2} at the start of step n.
template <typename real>
__global__ void __launch_bounds__(128)
k_probe(const InstDev<real>* __restrict__ insts, DevState* st) {
    const InstDev<real>& I = insts[blockIdx.y];
    __shared__ double2 ph[2][MAXF];
    const long long n = st->step;
    const int buf = st->cur;
    const double dt = I.dt;
    for (int f = threadIdx.x; f < I.n_freq; f += blockDim.x) {
        double s, c;
        const double fr = I.freqs[f];
        sincospi(2.0 * fr * ((double)n * dt), &s, &c);
        ph[0][f] = make_double2(c * dt, s * dt);
        sincospi(2.0 * fr * (((double)n - 0.5) * dt), &s, &c);
        ph[1][f] = make_double2(c * dt, s * dt);
    }
    __syncthreads();
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= I.n_probe) return;
    const int comp = I.probe_comp[p];
    const real* F = I.F[buf][comp];
    double v = 0.0;
#pragma unroll
    for (int m = 0; m < 8; ++m) {
        const long long idx = I.probe_idx[8 * p + m];
        if (idx >= 0) v += I.probe_w[8 * p + m] * (double)F[idx];
    }
    const int ms = I.probe_mon[p];
    if (ms >= 0 && (n % I.save_span) == 0) monitor_store(I, n, ms, v, st);
    const int ds = I.probe_dft[p];
    if (ds >= 0) {
        double2* row = I.dft + (long long)ds * I.n_freq;
        const double2* pf = ph[comp >= 3 ? 1 : 0];
        for (int f = 0; f < I.n_freq; ++f) {
            double2 a = row[f];
            a.x += v * pf[f].x;
            a.y += v * pf[f].y;
            row[f] = a;
        }
    }
}

// --------------------------------------------------------------- split schedule
// Two passes per step over the current buffer, in place: H^{n+1/2} from E^n, then
// E^{n+1} from H^{n+1/2}.  Block = 32 x 8 threads over (x, y) at one z.
template <typename real>
__global__ void __launch_bounds__(256, 4)
k_split_h(const InstDev<real>* __restrict__ insts, const long long* __restrict__ blk0, int n_inst,
          DevState* st) {
    const long long b = blockIdx.x;
    const int ii = find_inst(blk0, n_inst, b);
    __shared__ __align__(16) InstDev<real> I;
    load_inst(insts + ii, &I);
    const long long lb = b - blk0[ii];
    const int bx = (I.nx + 31) >> 5, by = (I.ny + 7) >> 3;
    const int k = (int)(lb / (bx * by));
    const int rem = (int)(lb % (bx * by));
    const int j = (rem / bx) * 8 + threadIdx.y;
    const int i = (rem % bx) * 32 + threadIdx.x;
    const long long n = st->step;
    if (i >= I.nx || j >= I.ny) return;
    const int cur = st->cur;  // (H pass: no block-wide sync after this point)
    const long long o = (long long)k * I.plane + (long long)j * I.px + i;
    const real* Ex = I.F[cur][0];
    const real* Ey = I.F[cur][1];
    const real* Ez = I.F[cur][2];
    real* Hx = I.F[cur][3];
    real* Hy = I.F[cur][4];
    real* Hz = I.F[cur][5];
    const bool xi = i + 1 < I.nx, yj = j + 1 < I.ny, zk = k + 1 < I.nz;
    const real ex = Ex[o], ey = Ey[o], ez = Ez[o];
    const real ex_j = yj ? Ex[o + I.px] : real(0), ex_k = zk ? Ex[o + I.plane] : real(0);
    const real ey_i = xi ? Ey[o + 1] : real(0), ey_k = zk ? Ey[o + I.plane] : real(0);
    const real ez_i = xi ? Ez[o + 1] : real(0), ez_j = yj ? Ez[o + I.px] : real(0);
    real* const* psi = I.psiH[cur];
    {
        const real cv = curl_psi<real, 0, true>(I, i, j, k, o, ez_j - ez, ey_k - ey, psi, psi);
        real acc = -(I.S * cv);
        if (I.n_src) acc = apply_sources(I, SJ_HX, i, j, k, n, acc);
        Hx[o] = Hx[o] + acc;
    }
    {
        const real cv = curl_psi<real, 1, true>(I, i, j, k, o, ex_k - ex, ez_i - ez, psi, psi);
        real acc = -(I.S * cv);
        if (I.n_src) acc = apply_sources(I, SJ_HY, i, j, k, n, acc);
        Hy[o] = Hy[o] + acc;
    }
    {
        const real cv = curl_psi<real, 2, true>(I, i, j, k, o, ey_i - ey, ex_j - ex, psi, psi);
        real acc = -(I.S * cv);
        if (I.n_src) acc = apply_sources(I, SJ_HZ, i, j, k, n, acc);
        Hz[o] = Hz[o] + acc;
    }
}

template <typename real>
__global__ void __launch_bounds__(256, 4)
k_split_e(const InstDev<real>* __restrict__ insts, const long long* __restrict__ blk0, int n_inst,
          DevState* st) {
    const long long b = blockIdx.x;
    const int ii = find_inst(blk0, n_inst, b);
    __shared__ __align__(16) InstDev<real> I;
    load_inst(insts + ii, &I);
    const long long lb = b - blk0[ii];
    const int bx = (I.nx + 31) >> 5, by = (I.ny + 7) >> 3;
    const int k = (int)(lb / (bx * by));
    const int rem = (int)(lb % (bx * by));
    const int j = (rem / bx) * 8 + threadIdx.y;
    const int i = (rem % bx) * 32 + threadIdx.x;
    const long long n = st->step;
    if (i < I.nx && j < I.ny) {
        const int cur = st->cur;
        const long long o = (long long)k * I.plane + (long long)j * I.px + i;
        real* Ex = I.F[cur][0];
        real* Ey = I.F[cur][1];
        real* Ez = I.F[cur][2];
        const real* Hx = I.F[cur][3];
        const real* Hy = I.F[cur][4];
        const real* Hz = I.F[cur][5];
        const real hx = Hx[o], hy = Hy[o], hz = Hz[o];
        const real hx_j = j > 0 ? Hx[o - I.px] : real(0), hx_k = k > 0 ? Hx[o - I.plane] : real(0);
        const real hy_i = i > 0 ? Hy[o - 1] : real(0), hy_k = k > 0 ? Hy[o - I.plane] : real(0);
        const real hz_i = i > 0 ? Hz[o - 1] : real(0), hz_j = j > 0 ? Hz[o - I.px] : real(0);
        const int cb = I.combo[o];
        real* const* psi = I.psiE;
        {
            const real cv = curl_psi<real, 0, false>(I, i, j, k, o, hz - hz_j, hy - hy_k, psi, psi);
            Ex[o] = e_finish<real, 0>(I, i, j, k, n, cb, Ex[o], cv);
        }
        {
            const real cv = curl_psi<real, 1, false>(I, i, j, k, o, hx - hx_k, hz - hz_i, psi, psi);
            Ey[o] = e_finish<real, 1>(I, i, j, k, n, cb, Ey[o], cv);
        }
        {
            const real cv = curl_psi<real, 2, false>(I, i, j, k, o, hy - hy_i, hx - hx_j, psi, psi);
            Ez[o] = e_finish<real, 2>(I, i, j, k, n, cb, Ez[o], cv);
        }
    }
    finish_block(st);
}

// --------------------------------------------------------------- utilities
template <typename real>
__global__ void k_max_abs_e(InstDev<real> I, int buf, unsigned long long* out) {
    double m = 0.0;
    const long long total = (long long)I.nx * I.ny * I.nz;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
         t += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(t % I.nx);
        const long long r = t / I.nx;
        const int j = (int)(r % I.ny);
        const int k = (int)(r / I.ny);
        const long long o = (long long)k * I.plane + (long long)j * I.px + i;
        for (int c = 0; c < 3; ++c) {
            const double v = fabs((double)I.F[buf][c][o]);
            m = v > m ? v : m;
        }
    }
    for (int off = 16; off > 0; off >>= 1) {
        const double o2 = __shfl_down_sync(0xffffffffu, m, off);
        m = o2 > m ? o2 : m;
    }
    if ((threadIdx.x & 31) == 0) atomicMax(out, (unsigned long long)__double_as_longlong(m));
}

// --------------------------------------------------------------- launchers
template <typename real>
static long long split_blocks(const InstDev<real>& I) {
    return (long long)((I.nx + 31) / 32) * ((I.ny + 7) / 8) * I.nz;
}

template <typename real>
cudaError_t launch_probe(const InstDev<real>* d_insts, const InstDev<real>* h_insts, int n_inst,
                         DevState* st, cudaStream_t s) {
    int maxp = 0;
    for (int q = 0; q < n_inst; ++q) maxp = h_insts[q].n_probe > maxp ? h_insts[q].n_probe : maxp;
    if (maxp == 0) return cudaSuccess;
    dim3 grid((maxp + 127) / 128, n_inst);
    k_probe<real><<<grid, 128, 0, s>>>(d_insts, st);
    return cudaGetLastError();
}

// The block prefix of the split schedule (n_inst + 1 entries) is stored in
// device memory right after the instance table.
template <typename real>
cudaError_t launch_split_step(const InstDev<real>* d_insts, const InstDev<real>* h_insts,
                              int n_inst, DevState* st, cudaStream_t s) {
    cudaError_t e = launch_probe(d_insts, h_insts, n_inst, st, s);
    if (e != cudaSuccess) return e;
    long long total = 0;
    for (int q = 0; q < n_inst; ++q) total += split_blocks(h_insts[q]);
    const long long* blk0 = reinterpret_cast<const long long*>(d_insts + n_inst);
    dim3 block(32, 8);
    k_split_h<real><<<(unsigned)total, block, 0, s>>>(d_insts, blk0, n_inst, st);
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    k_split_e<real><<<(unsigned)total, block, 0, s>>>(d_insts, blk0, n_inst, st);
    return cudaGetLastError();
}

template <typename real>
cudaError_t launch_max_abs_e(const InstDev<real>& h_inst, int buf, double* d_out, cudaStream_t s) {
    cudaError_t e = cudaMemsetAsync(d_out, 0, sizeof(double), s);
    if (e != cudaSuccess) return e;
    k_max_abs_e<real><<<304, 256, 0, s>>>(h_inst, buf, reinterpret_cast<unsigned long long*>(d_out));
    return cudaGetLastError();
}

template cudaError_t launch_probe<double>(const InstDev<double>*, const InstDev<double>*, int,
                                          DevState*, cudaStream_t);
template cudaError_t launch_probe<float>(const InstDev<float>*, const InstDev<float>*, int,
                                         DevState*, cudaStream_t);
template cudaError_t launch_split_step<double>(const InstDev<double>*, const InstDev<double>*, int,
                                               DevState*, cudaStream_t);
template cudaError_t launch_split_step<float>(const InstDev<float>*, const InstDev<float>*, int,
                                              DevState*, cudaStream_t);
template cudaError_t launch_max_abs_e<double>(const InstDev<double>&, int, double*, cudaStream_t);
template cudaError_t launch_max_abs_e<float>(const InstDev<float>&, int, double*, cudaStream_t);

// split-schedule block counts, used by the host to size the prefix table
long long split_block_count_f64(const InstDev<double>& I) { return split_blocks(I); }
long long split_block_count_f32(const InstDev<float>& I) { return split_blocks(I); }

}  // namespace sj
