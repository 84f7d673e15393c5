// Fused single-pass leapfrog schedule.
//
// One launch per time step reads E^n, H^{n-1/2} (ping-pong buffer `cur`) and
// writes H^{n+1/2}, E^{n+1} (buffer cur^1) in one sweep, so each field
// component crosses HBM once in and once out per step.
//
// Work decomposition: a block owns a 32 x TY column tile of (x, y) and marches
// along z over one z segment.  For each plane k:
//   * E^n and H^{n-1/2} of plane k+3 (and its material-combo bytes) are
//     fetched by TMA (cp.async.bulk.tensor.3d) into a 3-slot shared-memory
//     ring, boxes starting at (i0-XOFF, j0-1) so the x/y halos arrive with
//     them (out-of-range coordinates read as zero = the domain's outside);
//   * main warps (ty < TY) update H of their own cells of plane k from the
//     ring, store them, and publish them in shared memory; the halo warp (ty == TY) recomputes H on the x-1 column and
//     y-1 row that E needs, without storing them (the neighbour tile owns them);
//   * main warps update E of plane k from the shared H plane and the own-cell
//     H of plane k-1 kept in registers, with CPML, sources and polarisation.
// A z segment starting at z0 > 0 first recomputes H of plane z0-1 (owned by
// the previous segment) to seed the k-1 registers.
// Extra blocks after the stepping blocks sample monitors and accumulate DFTs
// from buffer `cur`, which no block writes during the launch.
// Every wait on an mbarrier gives up after one second and records
// SJ_E_TIMEOUT in the device status instead of spinning forever.
#include <cuda.h>

#include "sj_physics.cuh"

namespace sj {

constexpr int FTX = 32;
constexpr int MAXF_FUSED = 256;
constexpr unsigned long long WAIT_NS = 1000000000ull;  // 1 s

template <typename real>
struct Box;
template <>
struct Box<float> {
    static constexpr int BX = 40, XOFF = 4;  // 160-byte rows, x0 = i0 - 4 (16-byte aligned)
};
template <>
struct Box<double> {
    static constexpr int BX = 36, XOFF = 2;  // 288-byte rows, x0 = i0 - 2 (16-byte aligned)
};

template <typename real, int TY, int NS>
struct Lay {
    static constexpr int BX = Box<real>::BX;
    static constexpr int XOFF = Box<real>::XOFF;
    static constexpr int RS = (int)sizeof(real);
    // per ring slot: E boxes (TY+2 rows from j0-1), H boxes (TY+1 rows from
    // j0-1), the combo box (TY rows of 32 bytes from (i0, j0))
    static constexpr int EBOXB = (TY + 2) * BX * RS;
    static constexpr int HBOXB = (TY + 1) * BX * RS;
    static constexpr int CBOXB = TY * 32;
    static constexpr int EBOXP = (EBOXB + 127) / 128 * 128;
    static constexpr int HBOXP = (HBOXB + 127) / 128 * 128;
    static constexpr int CBOXP = (CBOXB + 127) / 128 * 128;
    static constexpr int SLOT = 3 * EBOXP + 3 * HBOXP + CBOXP;
    static constexpr int TXB = 3 * EBOXB + 3 * HBOXB + CBOXB;     // bytes per plane
    static constexpr int RING = NS * SLOT;
    static constexpr int HW = FTX + 1;
    static constexpr int HPL = (TY + 1) * HW;                      // elements per H plane
    static constexpr int HB = (3 * HPL * RS + 127) / 128 * 128;
    static constexpr int MBAR = RING + HB;
    static constexpr int BYTES = MBAR + 8 * NS + 64;
    // blocks per SM the register budget aims for (shared memory permitting)
    static constexpr int MINB = (TY >= 16 || (RS == 8 && TY >= 8)) ? 2 : 3;
};

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ unsigned long long globaltimer() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count));
}

__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    return ok != 0;
}

// Bounded wait: false after WAIT_NS without completion.
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity) {
    if (mbar_try_wait(bar, parity)) return true;
    const unsigned long long t0 = globaltimer();
    while (!mbar_try_wait(bar, parity)) {
        if (globaltimer() - t0 > WAIT_NS) return false;
    }
    return true;
}

__device__ __forceinline__ void tma_load_3d(uint32_t dst, const void* tmap, int x, int y, int z,
                                            uint32_t bar) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes"
        " [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(dst),
        "l"(reinterpret_cast<uint64_t>(tmap)), "r"(x), "r"(y), "r"(z), "r"(bar)
        : "memory");
}

__device__ __forceinline__ int find_block(const long long* __restrict__ pre, int n, long long b) {
    int lo = 0, hi = n - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (pre[mid] <= b)
            lo = mid;
        else
            hi = mid - 1;
    }
    return lo;
}

// --------------------------------------------------------------- probe blocks
template <typename real>
__device__ void probe_block(const InstDev<real>& I, long long chunk, long long n, int buf,
                            DevState* st, double2* ph /* [2][MAXF_FUSED] */) {
    const int tid = threadIdx.y * blockDim.x + threadIdx.x;
    const double dt = I.dt;
    for (int f = tid; f < I.n_freq; f += blockDim.x * blockDim.y) {
        double s, c;
        const double fr = I.freqs[f];
        sincospi(2.0 * fr * ((double)n * dt), &s, &c);
        ph[f] = make_double2(c * dt, s * dt);
        sincospi(2.0 * fr * (((double)n - 0.5) * dt), &s, &c);
        ph[MAXF_FUSED + f] = make_double2(c * dt, s * dt);
    }
    __syncthreads();
    const long long p = chunk * (blockDim.x * blockDim.y) + tid;
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
    if (ms >= 0 && (n % I.save_span) == 0) {
        const long long s = n / I.save_span;
        if (s < I.mon_cap)
            I.mon[s * I.n_mon + ms] = v;
        else
            st->status = SJ_E_RANGE;
    }
    const int ds = I.probe_dft[p];
    if (ds >= 0) {
        double2* row = I.dft + (long long)ds * I.n_freq;
        const double2* pf = ph + (comp >= 3 ? MAXF_FUSED : 0);
        for (int f = 0; f < I.n_freq; ++f) {
            double2 a = row[f];
            a.x += v * pf[f].x;
            a.y += v * pf[f].y;
            row[f] = a;
        }
    }
}

// --------------------------------------------------------------- stepping blocks
// Index of coordinate q inside the CPML slab storage of axis a, or -1.
template <typename real>
__device__ __forceinline__ int slab_q(const InstDev<real>& I, int a, int q) {
    const int n = a == 0 ? I.nx : (a == 1 ? I.ny : I.nz);
    const int pl = I.pl[a], ph = I.ph[a];
    return q < pl ? q : (q >= n - ph ? q - (n - ph) + pl : -1);
}

// One CPML auxiliary term: psi = b psi + c d along axis A at cell (i, j, k)
// whose slab index along A is q (>= 0).  Returns the updated psi.
template <typename real, int A, bool HALF>
__device__ __forceinline__ real psi_term(const InstDev<real>& I, int slot, int i, int j, int k, int q,
                                         real d, real* const* pin, real* const* pout, bool store) {
    constexpr int BOFF = HALF ? 2 : 0;
    const int n = A == 0 ? I.nx : (A == 1 ? I.ny : I.nz);
    const int w = I.pl[A] + I.ph[A];
    const int c = A == 0 ? i : (A == 1 ? j : k);
    long long o;
    if (A == 0)
        o = ((long long)k * I.ny + j) * w + q;
    else if (A == 1)
        o = ((long long)k * w + q) * I.px + i;
    else
        o = ((long long)q * I.ny + j) * I.px + i;
    o += (long long)slot * I.slabvol[A];
    const real psi = I.prof[A][BOFF * n + c] * pin[A][o] + I.prof[A][(BOFF + 1) * n + c] * d;
    if (store) pout[A][o] = psi;
    return psi;
}

// curl of component CA with its CPML terms; xq/yq/zq = slab indices (-1 = none).
// Same operation order as curl_psi: cur = d1 - d2; += psi(A1); -= psi(A2).
template <typename real, int CA, bool HALF>
__device__ __forceinline__ real curl_q(const InstDev<real>& I, int i, int j, int k, int xq, int yq, int zq,
                                       real d1, real d2, real* const* pin, real* const* pout, bool store) {
    constexpr int A1 = (CA + 1) % 3, A2 = (CA + 2) % 3;
    constexpr int P1 = (CA > A1) ? CA - 1 : CA;
    constexpr int P2 = (CA > A2) ? CA - 1 : CA;
    const int q1 = A1 == 0 ? xq : (A1 == 1 ? yq : zq);
    const int q2 = A2 == 0 ? xq : (A2 == 1 ? yq : zq);
    real cur = d1 - d2;
    if (q1 >= 0) cur += psi_term<real, A1, HALF>(I, P1, i, j, k, q1, d1, pin, pout, store);
    if (q2 >= 0) cur -= psi_term<real, A2, HALF>(I, P2, i, j, k, q2, d2, pin, pout, store);
    return cur;
}

template <typename real, int TY, int NS>
__device__ void step_block(const InstDev<real>& I, long long local, long long n, int cur, bool dry,
                           DevState* st, unsigned char* smem) {
    using L = Lay<real, TY, NS>;
    real* sH = reinterpret_cast<real*>(smem + L::RING);
    uint64_t* bars = reinterpret_cast<uint64_t*>(smem + L::MBAR);
    __shared__ int abort_flag;

    const int tx = threadIdx.x, ty = threadIdx.y;
    const bool lead = (tx == 0 && ty == 0);
    const int ntxy = I.f_ntx * I.f_nty;
    const int zseg = (int)(local / ntxy);
    const int rem = (int)(local % ntxy);
    const int i0 = (rem % I.f_ntx) * FTX;
    const int j0 = (rem / I.f_ntx) * TY;
    const int z0 = zseg * I.f_zs;
    const int z1 = min(I.nz, z0 + I.f_zs);
    const int kstart = z0 > 0 ? z0 - 1 : 0;
    const int kend = z1;  // planes kstart..kend are read (k+1 of the last plane z1-1)

    // tensor maps: [0..5] E[buffer][c], [6..11] H[buffer][c], [12] combo
    const unsigned char* tmE = static_cast<const unsigned char*>(I.tmap) + (size_t)cur * 3 * 128;
    const unsigned char* tmH = static_cast<const unsigned char*>(I.tmap) + (size_t)(6 + cur * 3) * 128;
    const unsigned char* tmC = static_cast<const unsigned char*>(I.tmap) + (size_t)12 * 128;
    if (lead) {
        abort_flag = 0;
        for (int q = 0; q < NS; ++q) mbar_init(smem_u32(&bars[q]), 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    __syncthreads();
    auto issue = [&](int p) {  // plane p into its slot (lead thread only)
        const int q = p - kstart;
        const int sl = q % NS;
        const uint32_t bar = smem_u32(&bars[sl]);
        unsigned char* base = smem + sl * L::SLOT;
        mbar_expect_tx(bar, (uint32_t)L::TXB);
        for (int c = 0; c < 3; ++c)
            tma_load_3d(smem_u32(base + c * L::EBOXP), tmE + c * 128, i0 - L::XOFF, j0 - 1, p, bar);
        for (int c = 0; c < 3; ++c)
            tma_load_3d(smem_u32(base + 3 * L::EBOXP + c * L::HBOXP), tmH + c * 128, i0 - L::XOFF, j0 - 1, p,
                        bar);
        tma_load_3d(smem_u32(base + 3 * L::EBOXP + 3 * L::HBOXP), tmC, i0, j0, p, bar);
    };
    if (lead)
        for (int p = kstart; p <= min(kend, kstart + NS - 1); ++p) issue(p);

    const real S = I.S;
    real* const* psiHin = I.psiH[cur];
    real* const* psiHout = I.psiH[cur ^ 1];
    real* const* psiE = I.psiE;
    real* Hout[3] = {I.F[cur ^ 1][3], I.F[cur ^ 1][4], I.F[cur ^ 1][5]};
    real* Eout[3] = {I.F[cur ^ 1][0], I.F[cur ^ 1][1], I.F[cur ^ 1][2]};

    const bool main = ty < TY;
    const int i = i0 + tx, j = j0 + ty;
    const bool own = main && i < I.nx && j < I.ny;
    // halo cells of the halo warp: y-1 row (hr) and x-1 column (hc)
    const int hri = i0 + tx, hrj = j0 - 1;
    const int hci = i0 - 1, hcj = j0 + tx;
    const bool hrow = !main && hrj >= 0 && hri < I.nx;
    const bool hcol = !main && tx < TY && hci >= 0 && hcj < I.ny;
    // CPML slab indices along x and y, fixed for the whole z march
    const int xq = slab_q(I, 0, i), yq = slab_q(I, 1, j);
    const int xq_r = slab_q(I, 0, hri), yq_r = slab_q(I, 1, hrj);
    const int xq_c = slab_q(I, 0, hci), yq_c = slab_q(I, 1, hcj);
    // sources overlapping this tile's footprint (own cells and halo), one bit per source
    unsigned smask = 0;
    for (int q = 0; q < I.n_src; ++q) {
        const SrcDev<real>& sv = I.src[q];
        if (sv.lo[0] < i0 + FTX && sv.lo[0] + sv.n[0] > i0 - 1 && sv.lo[1] < j0 + TY &&
            sv.lo[1] + sv.n[1] > j0 - 1)
            smask |= 1u << q;
    }

    real hx_prev = 0, hy_prev = 0;  // H^{n+1/2} of plane k-1 at the own cell
    bool ok = true;

    auto E = [&](int slot, int c, int yy, int xx) -> real {  // E^n, y from j0-1, x from i0-XOFF
        return *reinterpret_cast<const real*>(smem + slot * L::SLOT + c * L::EBOXP +
                                              (yy * L::BX + xx) * L::RS);
    };
    auto HO = [&](int slot, int c, int yy, int xx) -> real {  // H^{n-1/2}, same origin
        return *reinterpret_cast<const real*>(smem + slot * L::SLOT + 3 * L::EBOXP + c * L::HBOXP +
                                              (yy * L::BX + xx) * L::RS);
    };
    auto CB = [&](int slot, int yy, int xx) -> int {  // combo, y from j0, x from i0
        return smem[slot * L::SLOT + 3 * L::EBOXP + 3 * L::HBOXP + yy * 32 + xx];
    };
    auto HS = [&](int c, int yy, int xx) -> real& { return sH[c * L::HPL + yy * L::HW + xx]; };

    for (int k = kstart; k < kend; ++k) {
        const int q = k - kstart;
        const int s0 = q % NS, s1 = (q + 1) % NS;
        const bool storing = k >= z0;
        const int zq = slab_q(I, 2, k);
        // sources that touch this plane (block-uniform)
        unsigned pm = 0;
        for (unsigned m = smask; m; m &= m - 1) {
            const int qq = __ffs(m) - 1;
            const SrcDev<real>& sv = I.src[qq];
            if (k >= sv.lo[2] && k < sv.lo[2] + sv.n[2]) pm |= 1u << qq;
        }
        // wait for planes k and k+1
        if (q == 0) ok &= mbar_wait(smem_u32(&bars[s0]), (q / NS) & 1);
        ok &= mbar_wait(smem_u32(&bars[s1]), ((q + 1) / NS) & 1);
        if (!ok) abort_flag = 1;

        // ---------------- H phase
        const int yy = ty + 1, xe = tx + L::XOFF;
        if (own) {
            const long long o = (long long)k * I.plane + (long long)j * I.px + i;
            const real ex = E(s0, 0, yy, xe), ey = E(s0, 1, yy, xe), ez = E(s0, 2, yy, xe);
            const real ex_j = E(s0, 0, yy + 1, xe), ex_k = E(s1, 0, yy, xe);
            const real ey_i = E(s0, 1, yy, xe + 1), ey_k = E(s1, 1, yy, xe);
            const real ez_i = E(s0, 2, yy, xe + 1), ez_j = E(s0, 2, yy + 1, xe);
            const bool st_psi = storing && !dry;
            real hx, hy;
            {
                const real cv = curl_q<real, 0, true>(I, i, j, k, xq, yq, zq, ez_j - ez, ey_k - ey, psiHin,
                                                      psiHout, st_psi);
                real acc = -(S * cv);
                if (pm) acc = apply_sources(I, SJ_HX, i, j, k, n, acc);
                hx = HO(s0, 0, yy, xe) + acc;
            }
            {
                const real cv = curl_q<real, 1, true>(I, i, j, k, xq, yq, zq, ex_k - ex, ez_i - ez, psiHin,
                                                      psiHout, st_psi);
                real acc = -(S * cv);
                if (pm) acc = apply_sources(I, SJ_HY, i, j, k, n, acc);
                hy = HO(s0, 1, yy, xe) + acc;
            }
            if (storing) {
                real hz;
                {
                    const real cv = curl_q<real, 2, true>(I, i, j, k, xq, yq, zq, ey_i - ey, ex_j - ex,
                                                          psiHin, psiHout, st_psi);
                    real acc = -(S * cv);
                    if (pm) acc = apply_sources(I, SJ_HZ, i, j, k, n, acc);
                    hz = HO(s0, 2, yy, xe) + acc;
                }
                Hout[0][o] = hx;
                Hout[1][o] = hy;
                Hout[2][o] = hz;
                HS(0, yy, tx + 1) = hx;
                HS(1, yy, tx + 1) = hy;
                HS(2, yy, tx + 1) = hz;
            } else {
                hx_prev = hx;
                hy_prev = hy;
            }
        } else if (main && storing) {
            HS(0, yy, tx + 1) = 0;
            HS(1, yy, tx + 1) = 0;
            HS(2, yy, tx + 1) = 0;
        }
        if (!main && storing) {
            // halo warp: y-1 row (Hx, Hz) ...
            {
                real hx = 0, hz = 0;
                if (hrow) {
                    const int xe2 = tx + L::XOFF;
                    const real ey = E(s0, 1, 0, xe2), ez = E(s0, 2, 0, xe2), ex = E(s0, 0, 0, xe2);
                    {
                        const real cv = curl_q<real, 0, true>(I, hri, hrj, k, xq_r, yq_r, zq, E(s0, 2, 1, xe2) - ez,
                                                              E(s1, 1, 0, xe2) - ey, psiHin, psiHout, false);
                        real acc = -(S * cv);
                        if (pm) acc = apply_sources(I, SJ_HX, hri, hrj, k, n, acc);
                        hx = HO(s0, 0, 0, xe2) + acc;
                    }
                    {
                        const real cv = curl_q<real, 2, true>(I, hri, hrj, k, xq_r, yq_r, zq,
                                                              E(s0, 1, 0, xe2 + 1) - ey, E(s0, 0, 1, xe2) - ex,
                                                              psiHin, psiHout, false);
                        real acc = -(S * cv);
                        if (pm) acc = apply_sources(I, SJ_HZ, hri, hrj, k, n, acc);
                        hz = HO(s0, 2, 0, xe2) + acc;
                    }
                }
                HS(0, 0, tx + 1) = hx;
                HS(2, 0, tx + 1) = hz;
            }
            // ... and x-1 column (Hy, Hz)
            if (tx < TY) {
                real hy = 0, hz = 0;
                if (hcol) {
                    const int y2 = tx + 1, xe2 = L::XOFF - 1;
                    const real ex = E(s0, 0, y2, xe2), ey = E(s0, 1, y2, xe2), ez = E(s0, 2, y2, xe2);
                    {
                        const real cv = curl_q<real, 1, true>(I, hci, hcj, k, xq_c, yq_c, zq, E(s1, 0, y2, xe2) - ex,
                                                              E(s0, 2, y2, xe2 + 1) - ez, psiHin, psiHout, false);
                        real acc = -(S * cv);
                        if (pm) acc = apply_sources(I, SJ_HY, hci, hcj, k, n, acc);
                        hy = HO(s0, 1, y2, xe2) + acc;
                    }
                    {
                        const real cv = curl_q<real, 2, true>(I, hci, hcj, k, xq_c, yq_c, zq,
                                                              E(s0, 1, y2, xe2 + 1) - ey, E(s0, 0, y2 + 1, xe2) - ex,
                                                              psiHin, psiHout, false);
                        real acc = -(S * cv);
                        if (pm) acc = apply_sources(I, SJ_HZ, hci, hcj, k, n, acc);
                        hz = HO(s0, 2, y2, xe2) + acc;
                    }
                }
                HS(1, tx + 1, 0) = hy;
                HS(2, tx + 1, 0) = hz;
            }
        }
        __syncthreads();

        // ---------------- E phase
        if (own && storing) {
            const long long o = (long long)k * I.plane + (long long)j * I.px + i;
            const int xh = tx + 1;
            const real hx = HS(0, yy, xh), hy = HS(1, yy, xh), hz = HS(2, yy, xh);
            const real hx_j = HS(0, yy - 1, xh), hz_j = HS(2, yy - 1, xh);
            const real hy_i = HS(1, yy, xh - 1), hz_i = HS(2, yy, xh - 1);
            const int cb = CB(s0, ty, tx);
            const bool st_in = !dry;
            const bool src_e = pm != 0;
            {
                const real cv = curl_q<real, 0, false>(I, i, j, k, xq, yq, zq, hz - hz_j, hy - hy_prev, psiE, psiE, st_in);
                Eout[0][o] = e_finish<real, 0>(I, i, j, k, n, cb, E(s0, 0, yy, xe), cv, st_in, src_e);
            }
            {
                const real cv = curl_q<real, 1, false>(I, i, j, k, xq, yq, zq, hx - hx_prev, hz - hz_i, psiE, psiE, st_in);
                Eout[1][o] = e_finish<real, 1>(I, i, j, k, n, cb, E(s0, 1, yy, xe), cv, st_in, src_e);
            }
            {
                const real cv = curl_q<real, 2, false>(I, i, j, k, xq, yq, zq, hy - hy_i, hx - hx_j, psiE, psiE, st_in);
                Eout[2][o] = e_finish<real, 2>(I, i, j, k, n, cb, E(s0, 2, yy, xe), cv, st_in, src_e);
            }
            hx_prev = hx;
            hy_prev = hy;
        }
        __syncthreads();
        if (abort_flag) break;
        // slot s0 is free: fetch plane k + NS into it
        if (lead && k + NS <= kend) issue(k + NS);
    }
    if (abort_flag) {
        if (lead) {
            st->status = SJ_E_TIMEOUT;
            // bounded wait for every copy this block may still have in flight
            for (int q = 0; q < NS; ++q) mbar_wait(smem_u32(&bars[q]), 0), mbar_wait(smem_u32(&bars[q]), 1);
        }
        __syncthreads();
    }
}

template <typename real, int TY, int NS>
__global__ void __launch_bounds__(FTX * (TY + 1), (Lay<real, TY, NS>::MINB))
k_fused(const InstDev<real>* __restrict__ insts, int n_inst, DevState* st, FusedLaunch fl) {
    extern __shared__ __align__(128) unsigned char smem[];
    // the instance descriptor lives in shared memory for the whole block, so
    // its fields are re-read from there instead of pinning registers
    __shared__ __align__(16) InstDev<real> sI;
    const long long n = st->step;
    const int cur = st->cur;
    const long long b = blockIdx.x;
    const bool stepping = b < fl.n_items;
    const long long* pre = stepping ? fl.d_item_pre : fl.d_probe_pre;
    const long long lb = stepping ? b : b - fl.n_items;
    const int ii = find_block(pre, n_inst, lb);
    {
        const int* src = reinterpret_cast<const int*>(insts + ii);
        int* dst = reinterpret_cast<int*>(&sI);
        const int nw = (int)(sizeof(InstDev<real>) / sizeof(int));
        for (int w = threadIdx.y * blockDim.x + threadIdx.x; w < nw; w += blockDim.x * blockDim.y)
            dst[w] = src[w];
    }
    __syncthreads();
    if (stepping)
        step_block<real, TY, NS>(sI, lb - pre[ii], n, cur, fl.dry != 0, st, smem);
    else if (!fl.dry)
        probe_block<real>(sI, lb - pre[ii], n, cur, st, reinterpret_cast<double2*>(smem));
    // the last block to finish advances the step and flips the buffers
    __syncthreads();
    if (threadIdx.x == 0 && threadIdx.y == 0) {
        __threadfence();
        const unsigned prev = atomicAdd(&st->done, 1u);
        if (prev == gridDim.x - 1) {
            if (!fl.dry) {
                st->step += 1;
                st->cur ^= 1;
            }
            st->done = 0;
            __threadfence();
        }
    }
}

template <typename real, int TY, int NS>
static cudaError_t launch_ty(const InstDev<real>* d, int n_inst, DevState* st, const FusedLaunch& fl,
                             cudaStream_t s) {
    using L = Lay<real, TY, NS>;
    const int bytes = L::BYTES > 2 * MAXF_FUSED * 16 ? L::BYTES : 2 * MAXF_FUSED * 16;
    static bool attr = false;
    if (!attr) {
        cudaError_t e =
            cudaFuncSetAttribute(k_fused<real, TY, NS>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
        if (e != cudaSuccess) return e;
        attr = true;
    }
    const long long blocks = fl.n_items + fl.n_probe_blocks;
    k_fused<real, TY, NS><<<(unsigned)blocks, dim3(FTX, TY + 1), bytes, s>>>(d, n_inst, st, fl);
    return cudaGetLastError();
}

template <typename real>
cudaError_t launch_fused_step(const InstDev<real>* d_insts, int n_inst, DevState* st,
                              const FusedLaunch& fl, cudaStream_t s) {
    const int key = fl.ty * 16 + fl.nslot;
    switch (key) {
        case 4 * 16 + 3: return launch_ty<real, 4, 3>(d_insts, n_inst, st, fl, s);
        case 8 * 16 + 3: return launch_ty<real, 8, 3>(d_insts, n_inst, st, fl, s);
        case 16 * 16 + 3: return launch_ty<real, 16, 3>(d_insts, n_inst, st, fl, s);
        case 4 * 16 + 5: return launch_ty<real, 4, 5>(d_insts, n_inst, st, fl, s);
        case 8 * 16 + 5: return launch_ty<real, 8, 5>(d_insts, n_inst, st, fl, s);
        case 16 * 16 + 5: return launch_ty<real, 16, 5>(d_insts, n_inst, st, fl, s);
        default: return cudaErrorInvalidValue;
    }
}

template <>
int fused_box_width<float>() { return Box<float>::BX; }
template <>
int fused_box_width<double>() { return Box<double>::BX; }
template <>
int fused_box_xoff<float>() { return Box<float>::XOFF; }
template <>
int fused_box_xoff<double>() { return Box<double>::XOFF; }
int fused_block_threads(int ty) { return FTX * (ty + 1); }

template cudaError_t launch_fused_step<double>(const InstDev<double>*, int, DevState*, const FusedLaunch&,
                                               cudaStream_t);
template cudaError_t launch_fused_step<float>(const InstDev<float>*, int, DevState*, const FusedLaunch&,
                                              cudaStream_t);
}  // namespace sj
