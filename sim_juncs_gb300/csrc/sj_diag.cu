// Diagnostics computed on the device with FP64 sums: the discrete leapfrog
// energy of an instance and the flux spectrum of a surface sampled by DFT
// probes.  Neither is on the stepping path; both read the state the stepping
// kernels leave.
#include "sj_physics.cuh"

namespace sj {

constexpr int DIAG_THREADS = 256;

// Block-wide FP64 sum; every thread passes its value, thread 0 gets the sum.
__device__ __forceinline__ double block_sum(double v) {
    __shared__ double part[DIAG_THREADS / 32];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    if (l == 0) part[w] = v;
    __syncthreads();
    v = 0.0;
    if (w == 0) {
        v = l < DIAG_THREADS / 32 ? part[l] : 0.0;
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    }
    return v;
}

// W^n = sum_E eps E^n E^n + sum_H H^{n-1/2} H^{n+1/2}, H^{n+1/2} formed here
// from the plain (no CPML, no source) H update H - S curl_fwd(E^n).  eps is
// the stepper's own: 1 / (its inverse-eps coefficient), the design region's
// per-voxel value inside it.  One block per (j, k) row stride; per-block
// partial sums, added in a fixed order by k_sum (deterministic).
template <typename real>
__global__ void __launch_bounds__(DIAG_THREADS) k_energy(const InstDev<real> I, int cur, double* partial) {
    const real* const* F = I.F[cur];
    const int nx = I.nx, ny = I.ny, nz = I.nz;
    const double S = (double)I.S;
    auto E = [&](int c, int i, int j, int k) -> double {
        return (i < nx && j < ny && k < nz) ? (double)F[c][(long long)k * I.plane + (long long)j * I.px + i] : 0.0;
    };
    double acc = 0.0;
    for (long long r = blockIdx.x; r < (long long)ny * nz; r += gridDim.x) {
        const int j = (int)(r % ny), k = (int)(r / ny);
        const long long o0 = (long long)k * I.plane + (long long)j * I.px;
        for (int i = threadIdx.x; i < nx; i += blockDim.x) {
            const long long o = o0 + i;
            const real* cf = I.coef + (long long)I.combo[o] * I.ncoef;
            const double e[3] = {(double)F[0][o], (double)F[1][o], (double)F[2][o]};
            bool in_des = false;
            long long d = 0;
            if (I.dinv) {
                const int u = i - I.des_lo[0], v = j - I.des_lo[1], w = k - I.des_lo[2];
                if ((unsigned)u < (unsigned)I.des_n[0] && (unsigned)v < (unsigned)I.des_n[1] &&
                    (unsigned)w < (unsigned)I.des_n[2]) {
                    in_des = true;
                    d = ((long long)w * I.des_n[1] + v) * I.des_n[0] + u;
                }
            }
            for (int c = 0; c < 3; ++c) {
                const double inv = (double)(in_des ? I.dinv[d] : cf[c]);
                acc += e[c] * e[c] / inv;
            }
            // H^{n+1/2}_ca = H^{n-1/2}_ca - S ((E_a2(+a1) - E_a2) - (E_a1(+a2) - E_a1))
            const double ex_j = E(0, i, j + 1, k), ex_k = E(0, i, j, k + 1);
            const double ey_i = E(1, i + 1, j, k), ey_k = E(1, i, j, k + 1);
            const double ez_i = E(2, i + 1, j, k), ez_j = E(2, i, j + 1, k);
            const double cx = (ez_j - e[2]) - (ey_k - e[1]);
            const double cy = (ex_k - e[0]) - (ez_i - e[2]);
            const double cz = (ey_i - e[1]) - (ex_j - e[0]);
            const double hx = (double)F[3][o], hy = (double)F[4][o], hz = (double)F[5][o];
            acc += hx * (hx - S * cx) + hy * (hy - S * cy) + hz * (hz - S * cz);
        }
    }
    const double s = block_sum(acc);
    if (threadIdx.x == 0) partial[blockIdx.x] = s;
}

__global__ void __launch_bounds__(DIAG_THREADS) k_sum(const double* partial, int n, double scale, double* out) {
    double v = 0.0;
    for (int q = threadIdx.x; q < n; q += blockDim.x) v += partial[q];
    v = block_sum(v);
    if (threadIdx.x == 0) *out = scale * v;
}

constexpr int ENERGY_BLOCKS = 608;  // 4 x 152 SMs

int energy_partials() { return ENERGY_BLOCKS; }

template <typename real>
cudaError_t launch_energy(const InstDev<real>& h_inst, int cur, double scale, double* d_partial, double* d_out,
                          cudaStream_t s) {
    k_energy<real><<<ENERGY_BLOCKS, DIAG_THREADS, 0, s>>>(h_inst, cur, d_partial);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    k_sum<<<1, DIAG_THREADS, 0, s>>>(d_partial, ENERGY_BLOCKS, scale, d_out);
    return cudaGetLastError();
}

// out[f] = dA * sum_p Re(E1 conj(H2) - E2 conj(H1)) at frequency f, the
// four DFT rows of point p at rows[4p .. 4p+3]; one block per frequency.
__global__ void __launch_bounds__(DIAG_THREADS) k_flux(const double2* __restrict__ dft, int n_freq,
                                                       const int* __restrict__ rows, int n_pts, double dA,
                                                       double* __restrict__ out) {
    const int f = blockIdx.x;
    double acc = 0.0;
    for (int p = threadIdx.x; p < n_pts; p += blockDim.x) {
        const double2 e1 = dft[(long long)rows[4 * p + 0] * n_freq + f];
        const double2 e2 = dft[(long long)rows[4 * p + 1] * n_freq + f];
        const double2 h1 = dft[(long long)rows[4 * p + 2] * n_freq + f];
        const double2 h2 = dft[(long long)rows[4 * p + 3] * n_freq + f];
        acc += (e1.x * h2.x + e1.y * h2.y) - (e2.x * h1.x + e2.y * h1.y);
    }
    const double s = block_sum(acc);
    if (threadIdx.x == 0) out[f] = dA * s;
}

cudaError_t launch_flux(const double2* d_dft, int n_freq, const int* d_rows, int n_pts, double dA, double* d_out,
                        cudaStream_t s) {
    if (n_freq <= 0) return cudaSuccess;
    k_flux<<<n_freq, DIAG_THREADS, 0, s>>>(d_dft, n_freq, d_rows, n_pts, dA, d_out);
    return cudaGetLastError();
}

template cudaError_t launch_energy<double>(const InstDev<double>&, int, double, double*, double*, cudaStream_t);
template cudaError_t launch_energy<float>(const InstDev<float>&, int, double, double*, double*, cudaStream_t);

}  // namespace sj
