// Fused single-pass leapfrog schedule.
//
// One launch per time step reads E^n, H^{n-1/2} (ping-pong buffer `cur`) and
// writes H^{n+1/2}, E^{n+1} (buffer cur^1) in one sweep, so each field
// component crosses HBM once in and once out per step.
//
// Work decomposition: a block owns a 32 x TY column tile of (x, y) and marches
// along z over one z segment; warp w < TY owns row j0+w, warp TY is the halo
// warp.  The march is skewed by one plane: iteration h updates H of plane h
// and E of plane h-1, which read different (double-buffered) shared rows, so
// one barrier per plane suffices and the two updates overlap.
//   * Per-plane inputs arrive by TMA (cp.async.bulk.tensor.3d) in an NS-slot
//     shared-memory ring: E^n and H^{n-1/2} boxes from (i0-XOFF, j0-1), so the
//     x/y halos come with them (out-of-range coordinates read as zero, the
//     domain's outside), the combo bytes and, where the tile or plane touches
//     a CPML slab, that axis' psi_H tiles.
//   * H(h): main warps from the ring; the halo warp recomputes H on the y-1
//     row and x-1 column (owned by neighbour tiles, not stored).  Own Hx/Hz go
//     to a shared row for the next warp's y-1 neighbour; x-1 neighbours are
//     exchanged by warp shuffle (lane 0 takes the halo column).
//   * E(h-1): from the shared rows of plane h-1, own H of planes h-1 and h-2
//     and E^n and the combo byte of the own cell kept in registers since the
//     previous iteration; psi_E of the own cell is read from global memory at
//     the top of the iteration, so the H work hides its latency.
// A z segment starting at z0 > 0 first recomputes H of plane z0-1 (owned by
// the previous segment), unstored.  Extra blocks after the stepping blocks
// sample monitors and accumulate DFTs from buffer `cur`, which no block writes
// during the launch.  Every wait on an mbarrier gives up after a limit (100 ms
// unless sj_set_wait_limit sets another) and records SJ_E_TIMEOUT in the
// device status instead of spinning forever; the block then waits, again
// bounded (100 ms), for the copies it still has in flight and returns.
#include <cuda.h>

#include "sj_physics.cuh"

namespace sj {

constexpr int FTX = 32;
constexpr int MAXF_FUSED = 256;
constexpr unsigned long long WAIT_NS = 100000000ull;  // 100 ms (a healthy copy takes microseconds)
constexpr int MAXC_SMEM = 16;       // combos whose coefficient rows are staged in shared memory
constexpr int NCOEF_MAX = 6 + 3 * MAXP;

// tensor-map slots of one instance
constexpr int TM_E = 0, TM_H = 6, TM_C = 12, TM_PE = 13, TM_PH = 19, TM_COUNT = 31;

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
    // j0-1), combo and psi_H boxes (own cells, from (i0, j0))
    static constexpr int EBOXB = (TY + 2) * BX * RS;
    static constexpr int HBOXB = (TY + 1) * BX * RS;
    static constexpr int CBOXB = TY * 32;
    static constexpr int OBOXB = TY * FTX * RS;
    static constexpr int EBOXP = (EBOXB + 127) / 128 * 128;
    static constexpr int HBOXP = (HBOXB + 127) / 128 * 128;
    static constexpr int CBOXP = (CBOXB + 127) / 128 * 128;
    static constexpr int OBOXP = (OBOXB + 127) / 128 * 128;
    static constexpr int OFF_H = 3 * EBOXP;
    static constexpr int OFF_C = OFF_H + 3 * HBOXP;
    static constexpr int OFF_PH = OFF_C + CBOXP;             // 6 psi_H boxes [axis][pair]
    static constexpr int SLOT = OFF_PH + 6 * OBOXP;
    static constexpr int TXB = 3 * EBOXB + 3 * HBOXB + CBOXB; // bytes per plane without psi
    static constexpr int TXPSI = 2 * OBOXB;                   // extra bytes per CPML axis
    static constexpr int RING = NS * SLOT;
    // shared H exchange, double-buffered by plane parity:
    // rows [2][TY+1][Hx, Hz][32] (index 0 = the y-1 halo row, w+1 = warp w),
    // halo column [2][Hy, Hz][TY]
    static constexpr int OFF_ROW = RING;
    static constexpr int OFF_COL = OFF_ROW + 2 * (TY + 1) * 2 * FTX * RS;
    static constexpr int OFF_PROF = OFF_COL + 2 * 2 * TY * RS;  // x [4][33], y [4][TY+1]
    static constexpr int PROF = 4 * (FTX + 1 + TY + 1) * RS;
    static constexpr int OFF_COEF = (OFF_PROF + PROF + 15) / 16 * 16;  // [MAXC_SMEM][NCOEF_MAX]
    static constexpr int OFF_FLAG = OFF_COEF + MAXC_SMEM * NCOEF_MAX * RS;
    static constexpr int MBAR = (OFF_FLAG + MAXC_SMEM + 15) / 16 * 16;
    static constexpr int BYTES = MBAR + 8 * NS;
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

// Bounded wait: false after limit_ns without completion.
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, unsigned long long limit_ns) {
    if (mbar_try_wait(bar, parity)) return true;
    const unsigned long long t0 = globaltimer();
    while (!mbar_try_wait(bar, parity)) {
        if (globaltimer() - t0 > limit_ns) return false;
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
    if (ms >= 0 && (n % I.save_span) == 0) monitor_store(I, n, ms, v, st);
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
// CPML state of one cell for one plane: per axis, slab membership and b, c.
template <typename real>
struct Cpml {
    bool on[3];
    real b[3], c[3];
};

// psi_old of the 6 [axis][pair] auxiliaries of one cell, either in registers
// (get(A, P) with compile-time indices) or in the shared ring.
template <typename real>
struct PsiRegs {
    real v[6];
    __device__ __forceinline__ real get(int a, int p) const { return v[a * 2 + p]; }
};
template <typename real>
struct PsiRing {
    const real* base;
    int stride;
    __device__ __forceinline__ real get(int a, int p) const { return base[(a * 2 + p) * stride]; }
};

// curl of component CA with its CPML terms; psi_new goes to global memory at
// offset o.  Same operation order as curl_psi: cur = d1 - d2; += psi(A1); -= psi(A2).
template <typename real, int CA, typename Psi>
__device__ __forceinline__ real curl_c(const Cpml<real>& cp, real d1, real d2, const Psi& pin,
                                       real* const* pout, long long o, long long vol, bool store) {
    constexpr int A1 = (CA + 1) % 3, A2 = (CA + 2) % 3;
    constexpr int P1 = (CA > A1) ? CA - 1 : CA;
    constexpr int P2 = (CA > A2) ? CA - 1 : CA;
    real cur = d1 - d2;
    if (cp.on[A1]) {
        const real psi = cp.b[A1] * pin.get(A1, P1) + cp.c[A1] * d1;
        if (store) pout[A1][P1 * vol + o] = psi;
        cur += psi;
    }
    if (cp.on[A2]) {
        const real psi = cp.b[A2] * pin.get(A2, P2) + cp.c[A2] * d2;
        if (store) pout[A2][P2 * vol + o] = psi;
        cur -= psi;
    }
    return cur;
}

template <typename real, int TY, int NS>
__device__ void step_block(const InstDev<real>& I, long long local, long long n, int cur, bool dry,
                           DevState* st, unsigned char* smem, unsigned long long wait_ns, bool stall) {
    using L = Lay<real, TY, NS>;
    real* sRow = reinterpret_cast<real*>(smem + L::OFF_ROW);   // [2][TY+1][Hx, Hz][32]
    real* sCol = reinterpret_cast<real*>(smem + L::OFF_COL);   // [2][Hy, Hz][TY]
    real* prof = reinterpret_cast<real*>(smem + L::OFF_PROF);  // [4][33] x, then [4][TY+1] y
    real* scoef = reinterpret_cast<real*>(smem + L::OFF_COEF);
    unsigned char* sflag = smem + L::OFF_FLAG;
    uint64_t* bars = reinterpret_cast<uint64_t*>(smem + L::MBAR);
    __shared__ int abort_flag;

    const int tx = threadIdx.x, w = threadIdx.y;
    const bool lead = (tx == 0 && w == 0);
    const int ntxy = I.f_ntx * I.f_nty;
    const int zseg = (int)(local / ntxy);
    const int rem = (int)(local % ntxy);
    const int i0 = (rem % I.f_ntx) * FTX;
    const int j0 = (rem / I.f_ntx) * TY;
    const int z0 = zseg * I.f_zs;
    const int z1 = min(I.nz, z0 + I.f_zs);
    const int kstart = z0 > 0 ? z0 - 1 : 0;
    const int kend = z1;  // H of planes kstart..kend-1 reads planes kstart..kend

    // does the tile (incl. its x-1 / y-1 halo) touch the x / y CPML slabs?
    const bool tile_x = (I.pl[0] > 0 && i0 - 1 < I.pl[0]) || (I.ph[0] > 0 && i0 + FTX - 1 >= I.nx - I.ph[0]);
    const bool tile_y = (I.pl[1] > 0 && j0 - 1 < I.pl[1]) || (I.ph[1] > 0 && j0 + TY - 1 >= I.ny - I.ph[1]);
    const bool have_z = I.pl[2] + I.ph[2] > 0;

    const unsigned char* tm = static_cast<const unsigned char*>(I.tmap);
    if (lead) {
        abort_flag = 0;
        for (int q = 0; q < NS; ++q) mbar_init(smem_u32(&bars[q]), 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    // CPML profiles of the tile's columns (i0-1 .. i0+31) and rows (j0-1 .. j0+TY-1),
    // and the combo table when it is small
    const bool coef_smem = I.n_combos <= MAXC_SMEM;
    {
        const int t = w * FTX + tx;
        const int nthr = FTX * (TY + 1);
        for (int q = t; q < 4 * (FTX + 1); q += nthr) {
            const int a = q / (FTX + 1), x = i0 - 1 + q % (FTX + 1);
            prof[q] = (x >= 0 && x < I.nx) ? I.prof[0][a * I.nx + x] : real(0);
        }
        for (int q = t; q < 4 * (TY + 1); q += nthr) {
            const int a = q / (TY + 1), y = j0 - 1 + q % (TY + 1);
            prof[4 * (FTX + 1) + q] = (y >= 0 && y < I.ny) ? I.prof[1][a * I.ny + y] : real(0);
        }
        if (coef_smem) {
            for (int q = t; q < I.n_combos * I.ncoef; q += nthr) scoef[q] = I.coef[q];
            for (int q = t; q < I.n_combos; q += nthr) sflag[q] = I.cflag[q];
        }
    }
    __syncthreads();
    const real* coef = coef_smem ? scoef : I.coef;
    const unsigned char* cflag = coef_smem ? sflag : I.cflag;

    auto in_z = [&](int p) { return have_z && (p < I.pl[2] || p >= I.nz - I.ph[2]); };
    auto issue = [&](int p, int sl) {  // plane p into ring slot sl (lead thread only)
        const uint32_t bar = smem_u32(&bars[sl]);
        unsigned char* base = smem + sl * L::SLOT;
        const bool pz = in_z(p);
        const uint32_t bytes = (uint32_t)(L::TXB + L::TXPSI * ((int)tile_x + (int)tile_y + (int)pz));
        mbar_expect_tx(bar, bytes);
        const int xh = i0 - L::XOFF, yh = j0 - 1;
        for (int c = 0; c < 3; ++c) {
            tma_load_3d(smem_u32(base + c * L::EBOXP), tm + (TM_E + cur * 3 + c) * 128, xh, yh, p, bar);
            tma_load_3d(smem_u32(base + L::OFF_H + c * L::HBOXP), tm + (TM_H + cur * 3 + c) * 128, xh, yh, p,
                        bar);
        }
        tma_load_3d(smem_u32(base + L::OFF_C), tm + TM_C * 128, i0, j0, p, bar);
        for (int a = 0; a < 3; ++a) {
            if (!(a == 0 ? tile_x : (a == 1 ? tile_y : pz))) continue;
            for (int pp = 0; pp < 2; ++pp)
                tma_load_3d(smem_u32(base + L::OFF_PH + (a * 2 + pp) * L::OBOXP),
                            tm + (TM_PH + cur * 6 + a * 2 + pp) * 128, i0, j0, p, bar);
        }
    };
    if (lead)
        for (int p = kstart; p <= min(kend, kstart + NS - 1); ++p) {
            // test hook (sj_set_test_stall): the plane after the first is never
            // fetched, so the first iteration's wait on it runs out
            if (stall && p == kstart + 1) continue;
            issue(p, p - kstart);
        }

    const real S = I.S;
    const long long vol = I.vol;
    real* const* psiHin = I.psiH[cur];
    real* const* psiHout = I.psiH[cur ^ 1];
    real* const* psiE = I.psiE;
    real* const Hx = I.F[cur ^ 1][3];
    real* const Hy = I.F[cur ^ 1][4];
    real* const Hz = I.F[cur ^ 1][5];
    real* const Ex = I.F[cur ^ 1][0];
    real* const Ey = I.F[cur ^ 1][1];
    real* const Ez = I.F[cur ^ 1][2];

    const bool main = w < TY;
    const int i = i0 + tx, j = j0 + w;
    const bool own = main && i < I.nx && j < I.ny;
    // halo cells of the halo warp: y-1 row (hr) and x-1 column (hc)
    const int hri = i0 + tx, hrj = j0 - 1;
    const int hci = i0 - 1, hcj = j0 + tx;
    const bool hrow = !main && hrj >= 0 && hri < I.nx;
    const bool hcol = !main && tx < TY && hci >= 0 && hcj < I.ny;
    const int xp = tx + 1, yp = w + 1;  // own cell's index in the shared profiles
    const bool xon = in_slab(I, 0, i), yon = in_slab(I, 1, j);
    const bool xon_r = in_slab(I, 0, hri), yon_r = in_slab(I, 1, hrj);
    const bool xon_c = in_slab(I, 0, hci), yon_c = in_slab(I, 1, hcj);
    const real* px = prof;                   // [4][FTX+1]
    const real* py = prof + 4 * (FTX + 1);   // [4][TY+1]
    const long long oij = (long long)j * I.px + i;
    const long long oij_r = (long long)hrj * I.px + hri;
    const long long oij_c = (long long)hcj * I.px + hci;
    // sources overlapping this tile's footprint (own cells and halo), one bit per source
    unsigned smask = 0;
    for (int q = 0; q < I.n_src; ++q) {
        const SrcDev<real>& sv = I.src[q];
        if (sv.lo[0] < i0 + FTX && sv.lo[0] + sv.n[0] > i0 - 1 && sv.lo[1] < j0 + TY &&
            sv.lo[1] + sv.n[1] > j0 - 1)
            smask |= 1u << q;
    }
    auto plane_sources = [&](int p) {
        unsigned pm = 0;
        for (unsigned m = smask; m; m &= m - 1) {
            const int qq = __ffs(m) - 1;
            const SrcDev<real>& sv = I.src[qq];
            if (p >= sv.lo[2] && p < sv.lo[2] + sv.n[2]) pm |= 1u << qq;
        }
        return pm;
    };

    constexpr int EB = L::EBOXP / L::RS, HBX = L::HBOXP / L::RS, OB = L::OBOXP / L::RS;
    // shared-memory element offsets inside a ring slot
    const int e_own = (w + 1) * L::BX + tx + L::XOFF;    // E / H boxes: own cell
    const int o_own = w * FTX + tx;                      // combo / psi_H boxes: own cell
    const int e_row = tx + L::XOFF;                      // halo row cell (box row 0)
    const int e_col = (tx + 1) * L::BX + L::XOFF - 1;    // halo column cell

    // registers carried across the skewed march
    real hx1 = 0, hy1 = 0, hz1 = 0;  // own H of the E plane e = h-1
    real hx2 = 0, hy2 = 0;           // own H of plane e-1
    real eo0 = 0, eo1 = 0, eo2 = 0;  // own E^n of plane e
    int cbe = 0;                     // own combo of plane e
    // psi registers: main warps keep psi_E of plane e in p0; the halo warp keeps
    // psi_H of plane h for its row cell in p0 and its column cell in p1
    PsiRegs<real> p0, p1;
#pragma unroll
    for (int q = 0; q < 6; ++q) p0.v[q] = p1.v[q] = 0;
    bool zon_e = false;
    real bzi_e = 0, czi_e = 0;
    unsigned pm_e = 0;
    bool ok = true;
    int sa = 0, sb = 1 % NS;         // ring slots of planes h and h+1
    unsigned pa = 0, pb = (1 / NS) & 1;

    for (int h = kstart; h <= kend; ++h) {
        const bool do_h = h < kend;
        const bool store_h = h >= z0;            // H(h) is this segment's to store
        const bool do_e = h - 1 >= z0;           // E(h-1)
        const int q = h - kstart;
        const bool zon = in_z(h);
        real bzh = 0, czh = 0, bzi = 0, czi = 0;
        if (zon && do_h) {
            bzi = I.prof[2][h];
            czi = I.prof[2][I.nz + h];
            bzh = I.prof[2][2 * I.nz + h];
            czh = I.prof[2][3 * I.nz + h];
        }
        const unsigned pm = do_h ? plane_sources(h) : 0u;
        // global psi reads of this iteration, issued first so the H work hides them
        if (main) {
            if (do_e && own) {  // psi_E of the E plane (updated in place by its owner, us)
                const long long o = (long long)(h - 1) * I.plane + oij;
                if (xon) { p0.v[0] = psiE[0][o]; p0.v[1] = psiE[0][vol + o]; }
                if (yon) { p0.v[2] = psiE[1][o]; p0.v[3] = psiE[1][vol + o]; }
                if (zon_e) { p0.v[4] = psiE[2][o]; p0.v[5] = psiE[2][vol + o]; }
            }
        } else if (do_h && store_h) {  // halo psi_H (read-only: the neighbour tile owns it)
            const long long op = (long long)h * I.plane;
            if (hrow) {
                const long long o = op + oij_r;
                if (xon_r) p0.v[1] = psiHin[0][vol + o];
                if (yon_r) { p0.v[2] = psiHin[1][o]; p0.v[3] = psiHin[1][vol + o]; }
                if (zon) p0.v[4] = psiHin[2][o];
            }
            if (hcol) {
                const long long o = op + oij_c;
                if (xon_c) { p1.v[0] = psiHin[0][o]; p1.v[1] = psiHin[0][vol + o]; }
                if (yon_c) p1.v[3] = psiHin[1][vol + o];
                if (zon) p1.v[5] = psiHin[2][vol + o];
            }
        }
        if (do_h) {
            if (q == 0) ok &= mbar_wait(smem_u32(&bars[sa]), pa, wait_ns);
            ok &= mbar_wait(smem_u32(&bars[sb]), pb, wait_ns);
            if (!ok) abort_flag = 1;
        }
        const real* E0 = reinterpret_cast<const real*>(smem + sa * L::SLOT);      // E of plane h
        const real* E1 = reinterpret_cast<const real*>(smem + sb * L::SLOT);      // E of plane h+1
        const real* H0 = reinterpret_cast<const real*>(smem + sa * L::SLOT + L::OFF_H);
        const real* PH = reinterpret_cast<const real*>(smem + sa * L::SLOT + L::OFF_PH);
        const unsigned char* CBX = smem + sa * L::SLOT + L::OFF_C;
        const long long o_plane = (long long)h * I.plane;
        real* rowb = sRow + (h & 1) * (TY + 1) * 2 * FTX;     // rows of plane h
        real* colb = sCol + (h & 1) * 2 * TY;
        const real* rowe = sRow + ((h - 1) & 1) * (TY + 1) * 2 * FTX;  // rows of plane h-1
        const real* cole = sCol + ((h - 1) & 1) * 2 * TY;

        // ---------------- H(h)
        real hx0 = 0, hy0 = 0, hz0 = 0;
        real eon0 = 0, eon1 = 0, eon2 = 0;
        int cbn = 0;
        if (do_h && own) {
            const long long o = o_plane + oij;
            const real* e = E0 + e_own;
            const real ex = e[0], ey = e[EB], ez = e[2 * EB];
            const real ex_j = e[L::BX], ey_i = e[EB + 1], ez_i = e[2 * EB + 1], ez_j = e[2 * EB + L::BX];
            const real ex_k = E1[e_own], ey_k = E1[EB + e_own];
            const bool st_psi = store_h && !dry;
            Cpml<real> cp;
            cp.on[0] = xon;
            cp.on[1] = yon;
            cp.on[2] = zon;
            cp.b[0] = px[2 * (FTX + 1) + xp];
            cp.c[0] = px[3 * (FTX + 1) + xp];
            cp.b[1] = py[2 * (TY + 1) + yp];
            cp.c[1] = py[3 * (TY + 1) + yp];
            cp.b[2] = bzh;
            cp.c[2] = czh;
            const PsiRing<real> pin{PH + o_own, OB};
            {
                const real cv = curl_c<real, 0>(cp, ez_j - ez, ey_k - ey, pin, psiHout, o, vol, st_psi);
                real acc = -(S * cv);
                if (pm) acc = apply_sources(I, SJ_HX, i, j, h, n, acc);
                hx0 = H0[e_own] + acc;
            }
            {
                const real cv = curl_c<real, 1>(cp, ex_k - ex, ez_i - ez, pin, psiHout, o, vol, st_psi);
                real acc = -(S * cv);
                if (pm) acc = apply_sources(I, SJ_HY, i, j, h, n, acc);
                hy0 = H0[HBX + e_own] + acc;
            }
            {
                const real cv = curl_c<real, 2>(cp, ey_i - ey, ex_j - ex, pin, psiHout, o, vol, st_psi);
                real acc = -(S * cv);
                if (pm) acc = apply_sources(I, SJ_HZ, i, j, h, n, acc);
                hz0 = H0[2 * HBX + e_own] + acc;
            }
            if (store_h) {
                Hx[o] = hx0;
                Hy[o] = hy0;
                Hz[o] = hz0;
                // inputs of E(h), used next iteration: E^n and the combo byte
                eon0 = ex;
                eon1 = ey;
                eon2 = ez;
                cbn = CBX[o_own];
            }
        }
        if (do_h && store_h) {
            if (main) {
                rowb[(w + 1) * 2 * FTX + tx] = hx0;
                rowb[((w + 1) * 2 + 1) * FTX + tx] = hz0;
            } else {
                // halo warp: y-1 row (Hx, Hz) ...
                real vx = 0, vz = 0;
                if (hrow) {
                    const real* e = E0 + e_row;
                    const real ex = e[0], ey = e[EB], ez = e[2 * EB];
                    Cpml<real> cp;
                    cp.on[0] = xon_r;
                    cp.on[1] = yon_r;
                    cp.on[2] = zon;
                    cp.b[0] = px[2 * (FTX + 1) + xp];
                    cp.c[0] = px[3 * (FTX + 1) + xp];
                    cp.b[1] = py[2 * (TY + 1)];
                    cp.c[1] = py[3 * (TY + 1)];
                    cp.b[2] = bzh;
                    cp.c[2] = czh;
                    const long long o = o_plane + oij_r;
                    {
                        const real cv = curl_c<real, 0>(cp, e[2 * EB + L::BX] - ez, E1[EB + e_row] - ey, p0,
                                                        psiHout, o, vol, false);
                        real acc = -(S * cv);
                        if (pm) acc = apply_sources(I, SJ_HX, hri, hrj, h, n, acc);
                        vx = H0[e_row] + acc;
                    }
                    {
                        const real cv = curl_c<real, 2>(cp, e[EB + 1] - ey, e[L::BX] - ex, p0, psiHout, o,
                                                        vol, false);
                        real acc = -(S * cv);
                        if (pm) acc = apply_sources(I, SJ_HZ, hri, hrj, h, n, acc);
                        vz = H0[2 * HBX + e_row] + acc;
                    }
                }
                rowb[tx] = vx;
                rowb[FTX + tx] = vz;
                // ... and x-1 column (Hy, Hz)
                if (tx < TY) {
                    real vy = 0, vz2 = 0;
                    if (hcol) {
                        const real* e = E0 + e_col;
                        const real ex = e[0], ey = e[EB], ez = e[2 * EB];
                        Cpml<real> cp;
                        cp.on[0] = xon_c;
                        cp.on[1] = yon_c;
                        cp.on[2] = zon;
                        cp.b[0] = px[2 * (FTX + 1)];
                        cp.c[0] = px[3 * (FTX + 1)];
                        cp.b[1] = py[2 * (TY + 1) + tx + 1];
                        cp.c[1] = py[3 * (TY + 1) + tx + 1];
                        cp.b[2] = bzh;
                        cp.c[2] = czh;
                        const long long o = o_plane + oij_c;
                        {
                            const real cv = curl_c<real, 1>(cp, E1[e_col] - ex, e[2 * EB + 1] - ez, p1, psiHout,
                                                            o, vol, false);
                            real acc = -(S * cv);
                            if (pm) acc = apply_sources(I, SJ_HY, hci, hcj, h, n, acc);
                            vy = H0[HBX + e_col] + acc;
                        }
                        {
                            const real cv = curl_c<real, 2>(cp, e[EB + 1] - ey, e[L::BX] - ex, p1, psiHout, o,
                                                            vol, false);
                            real acc = -(S * cv);
                            if (pm) acc = apply_sources(I, SJ_HZ, hci, hcj, h, n, acc);
                            vz2 = H0[2 * HBX + e_col] + acc;
                        }
                    }
                    colb[tx] = vy;
                    colb[TY + tx] = vz2;
                }
            }
        }
        // ---------------- E(h-1): shared rows/column of plane h-1 are complete
        // since the barrier that ended the previous iteration
        if (do_e && main) {
            const int e = h - 1;
            // x-1 neighbours by shuffle (lane 0 takes the halo column)
            real hy_i = __shfl_up_sync(0xffffffffu, hy1, 1);
            real hz_i = __shfl_up_sync(0xffffffffu, hz1, 1);
            if (tx == 0) {
                hy_i = cole[w];
                hz_i = cole[TY + w];
            }
            // y-1 neighbours from the row above (the halo row for warp 0)
            const real hx_j = rowe[w * 2 * FTX + tx];
            const real hz_j = rowe[(w * 2 + 1) * FTX + tx];
            if (own) {
                const long long o = (long long)e * I.plane + oij;
                const real* cf = coef + cbe * I.ncoef;
                const bool disp = (cflag[cbe] & 1) != 0;
                const bool st_in = !dry;
                const bool src_e = pm_e != 0;
                Cpml<real> cp;
                cp.on[0] = xon;
                cp.on[1] = yon;
                cp.on[2] = zon_e;
                cp.b[0] = px[xp];
                cp.c[0] = px[(FTX + 1) + xp];
                cp.b[1] = py[yp];
                cp.c[1] = py[(TY + 1) + yp];
                cp.b[2] = bzi_e;
                cp.c[2] = czi_e;
                {
                    const real cv = curl_c<real, 0>(cp, hz1 - hz_j, hy1 - hy2, p0, psiE, o, vol, st_in);
                    Ex[o] = e_finish_row<real, 0>(I, i, j, e, n, cf, disp, eo0, cv, st_in, src_e);
                }
                {
                    const real cv = curl_c<real, 1>(cp, hx1 - hx2, hz1 - hz_i, p0, psiE, o, vol, st_in);
                    Ey[o] = e_finish_row<real, 1>(I, i, j, e, n, cf, disp, eo1, cv, st_in, src_e);
                }
                {
                    const real cv = curl_c<real, 2>(cp, hy1 - hy_i, hx1 - hx_j, p0, psiE, o, vol, st_in);
                    Ez[o] = e_finish_row<real, 2>(I, i, j, e, n, cf, disp, eo2, cv, st_in, src_e);
                }
            }
        }
        // shift the carried registers: plane h becomes the E plane
        hx2 = hx1;
        hy2 = hy1;
        hx1 = hx0;
        hy1 = hy0;
        hz1 = hz0;
        eo0 = eon0;
        eo1 = eon1;
        eo2 = eon2;
        cbe = cbn;
        zon_e = zon;
        bzi_e = bzi;
        czi_e = czi;
        pm_e = pm;
        __syncthreads();
        if (abort_flag) break;
        if (do_h) {
            // slot sa (plane h) is free: fetch plane h + NS into it
            if (lead && h + NS <= kend) issue(h + NS, sa);
            sa = sb;
            pa = pb;
            if (++sb == NS) sb = 0;
            pb = (unsigned)(((q + 2) / NS) & 1);
        }
    }
    if (abort_flag) {
        if (lead) {
            st->status = SJ_E_TIMEOUT;
            // bounded wait for every copy this block may still have in flight
            for (int qq = 0; qq < NS; ++qq)
                mbar_wait(smem_u32(&bars[qq]), 0, WAIT_NS), mbar_wait(smem_u32(&bars[qq]), 1, WAIT_NS);
        }
        __syncthreads();
    }
}

// Blocks per SM the register budget aims for.  FP64 steps are bound by the
// FP64 pipe rather than by latency, so they trade occupancy for no spills.
template <typename real, int TY>
struct MinBlocks {
    static constexpr int value = sizeof(real) == 8 ? (TY <= 4 ? 2 : 1) : (TY <= 4 ? 4 : (TY <= 8 ? 2 : 1));
};

template <typename real, int TY, int NS>
__global__ void __launch_bounds__(FTX * (TY + 1), MinBlocks<real, TY>::value)
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
        for (int q = threadIdx.y * blockDim.x + threadIdx.x; q < nw; q += blockDim.x * blockDim.y)
            dst[q] = src[q];
    }
    __syncthreads();
    if (stepping)
        step_block<real, TY, NS>(sI, lb - pre[ii], n, cur, fl.dry != 0, st, smem,
                                 fl.wait_ns ? fl.wait_ns : WAIT_NS, fl.stall != 0 && b == 0);
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
static cudaError_t launch_t(const InstDev<real>* d, int n_inst, DevState* st, const FusedLaunch& fl,
                            cudaStream_t s) {
    using L = Lay<real, TY, NS>;
    const int bytes = L::BYTES > 2 * MAXF_FUSED * 16 ? L::BYTES : 2 * MAXF_FUSED * 16;
    if (bytes > FUSED_MAX_SMEM) return cudaErrorInvalidConfiguration;
    static bool attr = false;
    if (!attr) {
        cudaError_t e = cudaFuncSetAttribute(k_fused<real, TY, NS>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
        if (e != cudaSuccess) return e;
        attr = true;
    }
    const long long blocks = fl.n_items + fl.n_probe_blocks;
    k_fused<real, TY, NS><<<(unsigned)blocks, dim3(FTX, TY + 1), bytes, s>>>(d, n_inst, st, fl);
    return cudaGetLastError();
}

// Supported tilings: (tile rows, TMA ring depth).
#define SJ_FUSED_TILINGS(X) X(4, 3) X(8, 3) X(16, 3) X(4, 4) X(8, 4)

template <typename real>
cudaError_t launch_fused_step(const InstDev<real>* d_insts, int n_inst, DevState* st,
                              const FusedLaunch& fl, cudaStream_t s) {
#define SJ_CASE(TYV, NV) \
    if (fl.ty == TYV && fl.ring == NV) return launch_t<real, TYV, NV>(d_insts, n_inst, st, fl, s);
    SJ_FUSED_TILINGS(SJ_CASE)
#undef SJ_CASE
    return cudaErrorInvalidValue;
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
int fused_tensor_maps() { return TM_COUNT; }

template <typename real>
int fused_smem_bytes(int ty, int ring) {
#define SJ_CASE(TYV, NV) \
    if (ty == TYV && ring == NV) return Lay<real, TYV, NV>::BYTES;
    SJ_FUSED_TILINGS(SJ_CASE)
#undef SJ_CASE
    return -1;
}
template int fused_smem_bytes<float>(int, int);
template int fused_smem_bytes<double>(int, int);

template cudaError_t launch_fused_step<double>(const InstDev<double>*, int, DevState*, const FusedLaunch&,
                                               cudaStream_t);
template cudaError_t launch_fused_step<float>(const InstDev<float>*, int, DevState*, const FusedLaunch&,
                                              cudaStream_t);
}  // namespace sj
