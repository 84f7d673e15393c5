// CEP and envelope extraction from monitor series, one CUDA block per series.
//
// Restates the reference's analysis class `signal` (scripts/phases.py:94-450)
// on its default path, as the sweeps call it (signal(t, v, lowpass_inc),
// get_envelope(), get_skewness()):
//   1. t0 guess: the |v|-weighted mean index of the local maxima of v^2
//      (_guess_t0_ind, :95-105; scipy.signal.find_peaks' plateau rule);
//   2. V = 2 rfft(v rolled by -t0); repeat: f0_ind = argmax |V|, f0 = the
//      trapezoid mean frequency of |V| below 2 f0_ind (_est_f0 'avg',
//      :225-228); a sinc low-pass of growing strength when f0 is above half
//      the band or |V| has a prominent peak above 3 f0 (is_noisy, :264-276),
//      at most MAX_LOWPASS_EVALS times (:313-341);
//   3. the band where |V| exceeds CUT_ALPHA of its value at f0 (_get_freq_fwhm,
//      :107-122), the unwrapped phase there (fix_angle_seq, :63-74) and its
//      linear regression: t0_corr = -slope / 2 pi, phi = intercept in
//      (-pi, pi]; recentred once when |t0_corr| > 2 / band (_param_est,
//      :124-153);
//   4. the envelope: |V| / (2 pi f) symmetrised about f0 (_get_sym_amps,
//      :357-375), the phase's odd-polynomial fit (get_ang_func, :239-260,
//      solved here as the linear least-squares problem curve_fit converges
//      to), inverse FFT rolled to the peak (calc_envelope, :377-429), and
//      its mean, width and skewness (get_mu/get_sig/get_skewness, :435-451).
// Transforms are direct sums in FP64 with exact integer phase reduction, one
// output bin per thread; the sequential scans run on thread 0.
#include "sj_internal.h"

namespace sj {

namespace {

constexpr int PH_THREADS = 128;
constexpr double PI = 3.141592653589793;
constexpr double CUT_ALPHA = 0.1;        // scripts/phases.py:24
constexpr double DIV_S = 4000.0;         // :17
constexpr int MAX_LOWPASS_EVALS = 4;     // :28
constexpr double NOISE_THRESH = 0.1;     // signal.__init__ default

struct Ctl {
    int t0_ind;         // current roll of the series
    int f0_ind;         // _est_f0's index
    int f_min, f_max;   // band [f_min, f_max)
    int go;             // loop control set by thread 0
    int status;
    int lowpass_steps;
    double f0, low_stren, last_cent;
    double t0_corr, phi;
    double poly[4];     // p1, p3, p5, p7 of the phase fit
};

// numpy's argmax: the first index of the largest value
__device__ int argmax(const double* a, int n) {
    int b = 0;
    for (int i = 1; i < n; ++i)
        if (a[i] > a[b]) b = i;
    return b;
}

// fix_angle (scripts/phases.py:51-61)
__device__ double fix_angle(double theta) {
    if (theta > PI) {
        theta -= 2 * PI * floor(theta / (2 * PI));
        if (theta > PI) theta -= 2 * PI;
    } else if (theta <= -PI) {
        theta += 2 * PI * (floor(-theta / (2 * PI)) + 1);
        if (theta > PI) theta -= 2 * PI;
    }
    return theta;
}

// fix_angle_seq (:63-74) in place: each angle moved by 2 pi when that brings
// it closer to the one before (the shift carries to every later angle)
__device__ void fix_angle_seq(double* a, int n) {
    for (int i = 1; i < n; ++i) {
        const double d = fabs(a[i] - a[i - 1]);
        double s = 0.0;
        if (fabs(a[i] + 2 * PI - a[i - 1]) < d)
            s = 2 * PI;
        else if (fabs(a[i] - 2 * PI - a[i - 1]) < d)
            s = -2 * PI;
        if (s != 0.0)
            for (int j = i; j < n; ++j) a[j] += s;
    }
}

// scipy.signal.find_peaks without conditions: local maxima, a flat top
// counted once at its middle (left of centre for an even width); the first
// and last samples are never peaks.  Calls f(index) per peak, in order.
template <typename F>
__device__ void local_maxima(const double* x, int n, F f) {
    int i = 1;
    const int i_max = n - 1;
    while (i < i_max) {
        if (x[i - 1] < x[i]) {
            int ahead = i + 1;
            while (ahead < i_max && x[ahead] == x[i]) ++ahead;
            if (x[ahead] < x[i]) {
                f((i + ahead - 1) / 2);
                i = ahead;
            }
        }
        ++i;
    }
}

// scipy.signal.peak_prominences with no window
__device__ double prominence(const double* x, int n, int peak) {
    double left_min = x[peak];
    for (int i = peak; i >= 0 && x[i] <= x[peak]; --i)
        if (x[i] < left_min) left_min = x[i];
    double right_min = x[peak];
    for (int i = peak; i <= n - 1 && x[i] <= x[peak]; ++i)
        if (x[i] < right_min) right_min = x[i];
    return x[peak] - fmax(left_min, right_min);
}

// numpy.trapz with unit spacing
__device__ double trapz(const double* y, int n) {
    double s = 0.0;
    for (int i = 0; i + 1 < n; ++i) s += (y[i] + y[i + 1]) / 2.0;
    return s;
}

__device__ __forceinline__ long long pmod(long long a, long long m) {
    const long long r = a % m;
    return r < 0 ? r + m : r;
}

// out[k] = 2 sum_m v[(m + shift) mod N] e^{-i 2 pi k m / N}, k < M (2 rfft of
// the rolled series), one bin per thread
__device__ void rfft2_rolled(const double* v, int N, int M, int shift, double2* out) {
    for (int k = threadIdx.x; k < M; k += blockDim.x) {
        double re = 0.0, im = 0.0;
        for (int m = 0; m < N; ++m) {
            const double x = v[pmod((long long)m + shift, N)];
            double s, c;
            sincospi(2.0 * (double)(((long long)k * m) % N) / (double)N, &s, &c);
            re += x * c;
            im -= x * s;
        }
        out[k] = make_double2(2.0 * re, 2.0 * im);
    }
}

// _apply_lowpass (:278-284): vf = vf0 sinc((f - cent) strength), v = the
// inverse real FFT (length L = 2 (M - 1)) rolled by t0, zero-padded to N
__device__ void apply_lowpass(const double2* vf0, int N, int M, double df, double cent, double strength,
                              int t0, double2* vf, double* mags, double* v) {
    for (int k = threadIdx.x; k < M; k += blockDim.x) {
        const double x = ((double)k * df - cent) * strength;
        const double y = PI * (x == 0.0 ? 1.0e-20 : x);
        const double s = sin(y) / y;
        const double2 a = vf0[k];
        vf[k] = make_double2(a.x * s, a.y * s);
        mags[k] = hypot(a.x * s, a.y * s);
    }
    __syncthreads();
    const int L = 2 * (M - 1);
    for (int n = threadIdx.x; n < N; n += blockDim.x) {
        if (n >= L) {
            v[n] = 0.0;
            continue;
        }
        const long long m = pmod((long long)n - t0, L);
        // x[m] = (Re X0 + Re X_{L/2} (-1)^m + 2 sum_{0<k<L/2} Re(X_k e^{i 2 pi k m / L})) / L
        double acc = vf[0].x + ((m & 1) ? -vf[M - 1].x : vf[M - 1].x);
        for (int k = 1; k < M - 1; ++k) {
            double s, c;
            sincospi(2.0 * (double)(((long long)k * m) % L) / (double)L, &s, &c);
            acc += 2.0 * (vf[k].x * c - vf[k].y * s);
        }
        v[n] = acc / (double)L;
    }
    __syncthreads();
}

// _get_freq_fwhm (:107-122)
__device__ void freq_band(const double* mags, int M, int f0i, double threshold, int* lo, int* hi) {
    const double cut = mags[f0i] * threshold;
    int f_min = f0i, f_max = f0i;
    const int jb = min(f0i, M - f0i - 1);
    for (int j = 0; j < jb; ++j) {
        if (mags[f0i - j] > cut) f_min = f0i - j - 1;
        if (mags[f0i + j] > cut) f_max = f0i + j + 1;
    }
    *lo = f_min;
    *hi = f_max;
}

// linregress of the unwrapped band phase against frequency (thread 0)
__device__ void band_regression(const double2* vf, int lo, int hi, double df, double* ang, double* slope,
                                double* intercept) {
    const int n = hi - lo;
    for (int i = 0; i < n; ++i) ang[i] = atan2(vf[lo + i].y, vf[lo + i].x);
    fix_angle_seq(ang, n);
    double xm = 0.0, ym = 0.0;
    for (int i = 0; i < n; ++i) xm += (double)(lo + i) * df, ym += ang[i];
    xm /= n;
    ym /= n;
    double sxx = 0.0, sxy = 0.0;
    for (int i = 0; i < n; ++i) {
        const double dx = (double)(lo + i) * df - xm;
        sxx += dx * dx;
        sxy += dx * (ang[i] - ym);
    }
    *slope = sxy / sxx;
    *intercept = ym - *slope * xm;
}

// u^k correctly rounded (double-double product, then one rounding), as the
// reference's numpy power gives it
__device__ double pow_int(double u, int k) {
    double hi = u, lo = 0.0;
    for (int i = 1; i < k; ++i) {
        const double p = __dmul_rn(hi, u);
        const double e = fma(hi, u, -p);                    // hi * u - p exactly
        const double l = __dadd_rn(__dmul_rn(lo, u), e);
        const double h2 = __dadd_rn(p, l);
        lo = __dadd_rn(l, -__dsub_rn(h2, p));
        hi = h2;
    }
    return hi;
}

// The phase model p7 u^7 + p5 u^5 + p3 u^3 + p1 u + p0, summed left to right
// without contraction, as the reference's lambda evaluates it.
__device__ double odd_model(const double* q, double u, double u3, double u5, double u7) {
    double m = __dmul_rn(q[4], u7);
    m = __dadd_rn(m, __dmul_rn(q[3], u5));
    m = __dadd_rn(m, __dmul_rn(q[2], u3));
    m = __dadd_rn(m, __dmul_rn(q[1], u));
    return __dadd_rn(m, q[0]);
}

// Least squares of angles ~ p0 + p1 u + p3 u^3 + p5 u^5 + p7 u^7, u = f - f0,
// by Householder QR (thread 0); a is scratch of 5 n doubles.  curve_fit
// starts from p = 1 and takes forward differences with step 2^-26 |p_j|
// (MINPACK's fdjac2); a parameter whose difference column is zero in every
// band bin (its term is lost to rounding) never moves from 1, so it is held
// at 1 here and the others are fitted to what remains.
__device__ void odd_poly_fit(const double* ang, int lo, int n, double df, double f0, double* a, double* poly) {
    constexpr int P = 5;
    double b[256];
    const double h = 1.4901161193847656e-08;  // sqrt(DBL_EPSILON)
    bool frozen[P] = {false, false, false, false, false};
    for (int j = 0; j < P; ++j) {
        double q[P] = {1.0, 1.0, 1.0, 1.0, 1.0};
        q[j] = 1.0 + h;
        const double one[P] = {1.0, 1.0, 1.0, 1.0, 1.0};
        bool zero = true;
        for (int i = 0; i < n && zero; ++i) {
            const double u = (double)(lo + i) * df - f0;
            const double u3 = pow_int(u, 3), u5 = pow_int(u, 5), u7 = pow_int(u, 7);
            zero = odd_model(q, u, u3, u5, u7) == odd_model(one, u, u3, u5, u7);
        }
        frozen[j] = zero;
    }
    int free_idx[P], nf = 0;
    for (int j = 0; j < P; ++j)
        if (!frozen[j]) free_idx[nf++] = j;
    for (int i = 0; i < n; ++i) {
        const double u = (double)(lo + i) * df - f0;
        const double col[P] = {1.0, u, pow_int(u, 3), pow_int(u, 5), pow_int(u, 7)};
        double y = ang[i];
        for (int j = 0; j < P; ++j)
            if (frozen[j]) y -= col[j];
        b[i] = y;
        for (int c = 0; c < nf; ++c) a[c * n + i] = col[free_idx[c]];
    }
    for (int c = 0; c < nf; ++c) {
        double nrm = 0.0;
        for (int i = c; i < n; ++i) nrm += a[c * n + i] * a[c * n + i];
        nrm = sqrt(nrm);
        const double alpha = a[c * n + c] > 0 ? -nrm : nrm;
        const double v0 = a[c * n + c] - alpha;
        // reflector v = (v0, a[c+1..]) with H = I - 2 v v^T / (v^T v)
        double vtv = v0 * v0;
        for (int i = c + 1; i < n; ++i) vtv += a[c * n + i] * a[c * n + i];
        if (vtv == 0.0) continue;
        for (int cc = c + 1; cc < nf; ++cc) {
            double d = v0 * a[cc * n + c];
            for (int i = c + 1; i < n; ++i) d += a[c * n + i] * a[cc * n + i];
            const double f = 2.0 * d / vtv;
            a[cc * n + c] -= f * v0;
            for (int i = c + 1; i < n; ++i) a[cc * n + i] -= f * a[c * n + i];
        }
        {
            double d = v0 * b[c];
            for (int i = c + 1; i < n; ++i) d += a[c * n + i] * b[i];
            const double f = 2.0 * d / vtv;
            b[c] -= f * v0;
            for (int i = c + 1; i < n; ++i) b[i] -= f * a[c * n + i];
        }
        a[c * n + c] = alpha;
    }
    double pf[P];
    for (int c = nf - 1; c >= 0; --c) {
        double s = b[c];
        for (int cc = c + 1; cc < nf; ++cc) s -= a[cc * n + c] * pf[cc];
        pf[c] = s / a[c * n + c];
    }
    double p[P] = {1.0, 1.0, 1.0, 1.0, 1.0};
    for (int c = 0; c < nf; ++c) p[free_idx[c]] = pf[c];
    poly[0] = p[1];
    poly[1] = p[2];
    poly[2] = p[3];
    poly[3] = p[4];
}

}  // namespace

// Per-series workspace layout, in doubles, for N samples (M = N / 2 + 1
// bins): every array starts on a 16-double (128-byte) boundary, so the
// double2 arrays are 16-byte aligned whatever N is.
struct PhaseLay {
    long long v0, v, vabs2, vf0, vf, mags, ef, vef, env, envt, scratch, total;
    __host__ __device__ explicit PhaseLay(int N) {
        const long long M = N / 2 + 1;
        auto al = [](long long x) { return (x + 15) & ~15LL; };
        v0 = 0;
        v = v0 + al(N);
        vabs2 = v + al(N);
        vf0 = vabs2 + al(N);
        vf = vf0 + al(2 * M);
        mags = vf + al(2 * M);
        ef = mags + al(M);
        vef = ef + al(N);
        env = vef + al(N);
        envt = env + al(2LL * N);
        scratch = envt + al(2LL * N);
        total = scratch + al(5 * 256 + 256);
    }
};

long long phase_workspace(int N) { return PhaseLay(N).total; }

// series q: v[q * s_series + k * s_sample], k < N; t[k] the sample times.
__global__ void __launch_bounds__(PH_THREADS)
k_phases(const double* __restrict__ vin, long long s_series, long long s_sample, int N, const double* __restrict__ t,
         double lowpass_inc, double* __restrict__ work, long long wstride, sj_phase_result* __restrict__ out) {
    __shared__ Ctl C;
    const int q = blockIdx.x;
    const int M = N / 2 + 1;
    const PhaseLay lay(N);
    double* w = work + (long long)q * wstride;  // wstride: a multiple of 16 doubles
    double* v0 = w + lay.v0;                    // original series
    double* v = w + lay.v;                      // v_pts
    double* vabs2 = w + lay.vabs2;              // v^2 (find_peaks input)
    double2* vf0 = reinterpret_cast<double2*>(w + lay.vf0);   // [M]
    double2* vf = reinterpret_cast<double2*>(w + lay.vf);     // [M]
    double* mags = w + lay.mags;                // [M]
    double* ef = w + lay.ef;                    // [N]
    double* vef = w + lay.vef;                  // [N]
    double2* env = reinterpret_cast<double2*>(w + lay.env);   // [N] Fourier envelope
    double2* envt = reinterpret_cast<double2*>(w + lay.envt); // [N] envelope
    double* scratch = w + lay.scratch;          // 5 * 256 + 256
    const double dt = t[1] - t[0];
    const double df = 1.0 / ((double)N * dt);  // rfftfreq spacing

    for (int k = threadIdx.x; k < N; k += blockDim.x) {
        const double x = vin[(long long)q * s_series + (long long)k * s_sample];
        v0[k] = x;
        v[k] = x;
        vabs2[k] = x * x;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        // _guess_t0_ind
        double at = 0.0, tm = 0.0;
        local_maxima(vabs2, N, [&](int i) {
            at += (double)i * fabs(v0[i]);
            tm += fabs(v0[i]);
        });
        C.t0_ind = tm <= 0.0 ? 0 : (int)(at / tm);
        C.status = 0;
        C.low_stren = 0.0;
        C.last_cent = 0.0;
        C.lowpass_steps = 0;
    }
    __syncthreads();
    rfft2_rolled(v, N, M, C.t0_ind, vf0);
    __syncthreads();
    for (int k = threadIdx.x; k < M; k += blockDim.x) {
        vf[k] = vf0[k];
        mags[k] = hypot(vf0[k].x, vf0[k].y);
    }
    __syncthreads();
    // the low-pass loop of signal.__init__
    for (;;) {
        if (threadIdx.x == 0) {
            C.go = 0;
            int fi = argmax(mags, M);
            const int L = min(2 * fi, M);
            double num = 0.0, den = 0.0;
            for (int i = 0; i + 1 < L; ++i) {
                num += (mags[i] * ((double)i * df) + mags[i + 1] * ((double)(i + 1) * df)) / 2.0;
                den += (mags[i] + mags[i + 1]) / 2.0;
            }
            const double f0 = num / den;
            const double r = rint(f0 / df);
            if (!isfinite(f0) || !(r < (double)M)) {
                C.status = SJ_PHASE_BAD_F0;
            } else {
                C.f0 = f0;
                C.f0_ind = (int)r;
                if (!(C.low_stren >= MAX_LOWPASS_EVALS * lowpass_inc)) {
                    double cent = -1.0;
                    if (C.f0_ind > M / 2) {
                        cent = 0.0;
                    } else {
                        // is_noisy: two or more peaks of prominence >= 0.1 |V(f0)|, one above 3 f0
                        const double pmin = NOISE_THRESH * mags[C.f0_ind];
                        int count = 0;
                        bool high = false;
                        local_maxima(mags, M, [&](int i) {
                            if (prominence(mags, M, i) >= pmin) {
                                ++count;
                                if (i > 3 * C.f0_ind) high = true;
                            }
                        });
                        if (count >= 2 && high) cent = (double)C.f0_ind * df / 2.0;
                    }
                    if (cent >= 0.0) {
                        C.low_stren += lowpass_inc;
                        C.last_cent = cent;
                        C.lowpass_steps += 1;
                        C.go = 1;
                    }
                }
            }
        }
        __syncthreads();
        if (C.status || !C.go) break;
        apply_lowpass(vf0, N, M, df, C.last_cent, C.low_stren, C.t0_ind, vf, mags, v);
    }
    // _param_est, recentred at most once
    // (the loop reads the control words only after a barrier: thread 0 writes
    // them at the top of a pass while the others wait)
    for (int pass = 0; pass < 2; ++pass) {
        if (threadIdx.x == 0 && !C.status) {
            C.go = 0;
            freq_band(mags, M, C.f0_ind, CUT_ALPHA, &C.f_min, &C.f_max);
            const int n = C.f_max - C.f_min;
            if (n == 0) {
                // the recentring test divides by the band width on every pass
                C.status = SJ_PHASE_EMPTY_BAND;
            } else {
                double slope, icpt;
                if (n > 256) {
                    C.status = SJ_PHASE_WIDE_BAND;
                } else {
                    band_regression(vf, C.f_min, C.f_max, df, scratch, &slope, &icpt);
                    C.t0_corr = -slope / (2 * PI);
                    C.phi = fix_angle(icpt);
                    if (pass == 0 && fabs(C.t0_corr) > 2.0 / (double)n) {
                        C.t0_ind += (int)(C.t0_corr / dt);
                        C.go = 1;
                    }
                }
            }
        }
        __syncthreads();
        if (C.status || !C.go) break;
        rfft2_rolled(v, N, M, C.t0_ind, env);  // env as scratch for the rolled spectrum
        __syncthreads();
        apply_lowpass(env, N, M, df, C.last_cent, C.low_stren, C.t0_ind, vf, mags, v);
    }
    // after a recentring, t_pts[t0_ind] must exist (Python indexing: -N <= t0_ind < N)
    if (threadIdx.x == 0 && !C.status && (C.t0_ind >= N || C.t0_ind < -N)) C.status = SJ_PHASE_BAD_T0;
    __syncthreads();
    if (C.status) {
        if (threadIdx.x == 0) {
            sj_phase_result r = {};
            r.f0 = C.f0;
            r.f0_ind = C.f0_ind;
            r.status = C.status;
            out[q] = r;
        }
        return;
    }
    // calc_envelope, symmetric mode
    if (threadIdx.x == 0) {
        int best = 0;  // t0_ind = argmax |v_pts|
        for (int i = 1; i < N; ++i)
            if (fabs(v[i]) > fabs(v[best])) best = i;
        C.t0_ind = best;
        for (int i = 0; i < N; ++i) ef[i] = vef[i] = 0.0;
        const double f0 = C.f0;
        // vec_vf = |V| / (2 pi f + exp(-DIV_S f / f0)), kept in envt's storage
        double* vec = reinterpret_cast<double*>(envt);
        for (int k = 0; k < M; ++k) {
            const double f = (double)k * df;
            vec[k] = mags[k] / (2 * PI * f + exp(-DIV_S * f / f0));
        }
        const int fi = (int)(f0 / df);
        const double lrp = f0 - fi * df;
        const int nn = min(fi, M - fi - 1);
        for (int i = 0; i < nn; ++i) {
            const double a = 0.5 * (vec[fi - i + 1] - vec[fi - i] + vec[fi + i + 1] - vec[fi + i]) * lrp / df +
                             0.5 * (vec[fi - i] + vec[fi + i]);
            vef[i] = a;
            const int ni = i == 0 ? 0 : N - i;
            vef[ni] = a;
            ef[ni] = 2 * PI * (f0 - (double)i * df) * vef[ni];
            ef[i] = 2 * PI * (f0 + (double)i * df) * vef[i];
        }
        // get_ang_func: the phase in the band fitted by an odd polynomial + constant
        freq_band(mags, M, C.f0_ind, CUT_ALPHA, &C.f_min, &C.f_max);
        const int n = C.f_max - C.f_min;
        if (n < 5 || n > 256) {
            C.status = n < 5 ? SJ_PHASE_NARROW_BAND : SJ_PHASE_WIDE_BAND;
        } else {
            for (int i = 0; i < n; ++i) scratch[i] = atan2(vf[C.f_min + i].y, vf[C.f_min + i].x);
            fix_angle_seq(scratch, n);
            odd_poly_fit(scratch, C.f_min, n, df, f0, scratch + 256, C.poly);
        }
    }
    __syncthreads();
    if (C.status) {
        if (threadIdx.x == 0) {
            sj_phase_result r = {};
            r.f0 = C.f0;
            r.phi = C.phi;
            r.t0_corr = C.t0_corr;
            r.f0_ind = C.f0_ind;
            r.band_lo = C.f_min;
            r.band_hi = C.f_max;
            r.lowpass_steps = C.lowpass_steps;
            r.status = C.status;
            out[q] = r;
        }
        return;
    }
    // env_fourier = ef e^{i vp(fftfreq)}, envelope = 2 roll(ifft(env_fourier), t0)
    for (int k = threadIdx.x; k < N; k += blockDim.x) {
        const int kk = k < (N + 1) / 2 ? k : k - N;  // fftfreq order
        const double x = (double)kk * df;
        const double x2 = x * x;
        const double ph = C.poly[3] * (x2 * x2 * x2 * x) + C.poly[2] * (x2 * x2 * x) + C.poly[1] * (x2 * x) +
                          C.poly[0] * x;
        double s, c;
        sincos(ph, &s, &c);
        env[k] = make_double2(ef[k] * c, ef[k] * s);
    }
    __syncthreads();
    for (int n = threadIdx.x; n < N; n += blockDim.x) {
        const long long m = pmod((long long)n - C.t0_ind, N);
        double re = 0.0, im = 0.0;
        for (int k = 0; k < N; ++k) {
            double s, c;
            sincospi(2.0 * (double)(((long long)k * m) % N) / (double)N, &s, &c);
            re += env[k].x * c - env[k].y * s;
            im += env[k].x * s + env[k].y * c;
        }
        envt[n] = make_double2(2.0 * re / N, 2.0 * im / N);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        // get_skewness on |envelope| normalised to unit area
        double* a = ef;   // reuse: |env|, then the moment integrands
        for (int i = 0; i < N; ++i) a[i] = hypot(envt[i].x, envt[i].y);
        const double area = trapz(a, N) * dt;
        for (int i = 0; i < N; ++i) a[i] = a[i] / area;
        for (int i = 0; i < N; ++i) vef[i] = a[i] * t[i];
        const double mu = trapz(vef, N) * dt;
        for (int i = 0; i < N; ++i) vef[i] = a[i] * ((t[i] - mu) * (t[i] - mu));
        const double sig = sqrt(trapz(vef, N) * dt);
        for (int i = 0; i < N; ++i) {
            const double d = t[i] - mu;
            vef[i] = a[i] * (d * d * d);
        }
        const double skew = trapz(vef, N) / (sig * sig * sig);
        // numpy's argmax of a complex array: largest real part, then imaginary
        int k = 0;
        for (int i = 1; i < N; ++i)
            if (envt[i].x > envt[k].x || (envt[i].x == envt[k].x && envt[i].y > envt[k].y)) k = i;
        sj_phase_result r = {};
        r.f0 = C.f0;
        r.phi = C.phi;
        r.t0_corr = C.t0_corr;
        r.t0 = t[C.t0_ind];
        r.amp[0] = envt[k].x;
        r.amp[1] = envt[k].y;
        r.mu = mu;
        r.sig = sig;
        r.skew = skew;
        r.f0_ind = C.f0_ind;
        r.band_lo = C.f_min;
        r.band_hi = C.f_max;
        r.lowpass_steps = C.lowpass_steps;
        r.status = 0;
        out[q] = r;
    }
}

cudaError_t launch_phases(const double* d_v, long long s_series, long long s_sample, int n_series, int N,
                          const double* d_t, double lowpass_inc, double* d_work, sj_phase_result* d_out,
                          cudaStream_t s) {
    if (n_series <= 0) return cudaSuccess;
    k_phases<<<n_series, PH_THREADS, 0, s>>>(d_v, s_series, s_sample, N, d_t, lowpass_inc, d_work,
                                             phase_workspace(N), d_out);
    return cudaGetLastError();
}

}  // namespace sj
