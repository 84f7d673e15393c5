// The spectrum save_field_times writes for each monitor series
// (src/disp.cpp:804, with the fft of src/data_utils.cpp:413-427): of N
// samples it takes the first N' = 2^floor(log2 N) and evaluates
//   F_k = sum_{m < N'} x_m e^{-i 2 pi m k / N},  k = -N'/2 .. N'/2 - 1,
// stored at index k mod N' (the phase step is 2 pi / N, not 2 pi / N').
// The reference does this O(N'^2) on the host per monitor; here one block
// row per monitor and one thread per output bin, FP64, with the phase m k
// reduced modulo N in integers before sincospi.
#include "sj_internal.h"

namespace sj {

namespace {

__global__ void k_spectrum(const double* __restrict__ mon, int n_mon, long long n, long long np, double* out) {
    const int ms = blockIdx.y;
    const long long kk = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (kk >= np) return;
    double sr = 0.0, si = 0.0;
    if (np > 1) {
        const long long k = kk < np / 2 ? kk : kk - np;
        for (long long m = 0; m < np; ++m) {
            const double x = mon[m * n_mon + ms];
            long long ph = (m * k) % n;
            if (ph < 0) ph += n;
            double s, c;
            sincospi(-2.0 * (double)ph / (double)n, &s, &c);
            sr += x * c;
            si += x * s;
        }
    }
    out[2 * ((long long)ms * np + kk)] = sr;
    out[2 * ((long long)ms * np + kk) + 1] = si;
}

}  // namespace

cudaError_t launch_spectrum(const double* d_mon, int n_mon, long long n, long long np, double* d_out, cudaStream_t s) {
    if (n_mon < 1 || np < 1) return cudaSuccess;
    const dim3 block(128), grid((unsigned)((np + 127) / 128), (unsigned)n_mon);
    k_spectrum<<<grid, block, 0, s>>>(d_mon, n_mon, n, np, d_out);
    return cudaGetLastError();
}

}  // namespace sj
