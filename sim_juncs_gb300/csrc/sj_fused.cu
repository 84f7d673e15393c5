// Fused single-pass leapfrog schedule.
//
// One launch per time step reads E^n, H^{n-1/2} (ping-pong buffer `cur`) and
// writes H^{n+1/2}, E^{n+1} (buffer cur^1) in one sweep, so each field
// component crosses HBM once in and once out per step.
//
// Work decomposition: a block owns a 32 x TY column tile of (x, y) and marches
// along z over one z segment.  For each plane k:
//   * every per-plane input of plane k+NS-1 is fetched by TMA
//     (cp.async.bulk.tensor.3d) into an NS-slot shared-memory ring: E^n and
//     H^{n-1/2} boxes starting at (i0-XOFF, j0-1) so the x/y halos arrive with
//     them (out-of-range coordinates read as zero = the domain's outside), the
//     material-combo bytes of the own cells and, where the tile or plane
//     touches a CPML slab, that axis' psi_H (own + halo) and psi_E (own) tiles;
//   * main warps (ty < TY) update H of their own cells of plane k from the
//     ring, store them, and publish them in shared memory; the halo warp
//     (ty == TY) recomputes H on the x-1 column and y-1 row that E needs,
//     without storing them (the neighbour tile owns them);
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

constexpr int NSLOT = 3;           // planes in the TMA ring (k, k+1 and one in flight)
constexpr int MAXC_SMEM = 16;       // combos whose coefficient rows are staged in shared memory
constexpr int NCOEF_MAX = 3 + 3 * MAXP;

// Tile = 32 x TY cells, TY = W * R: W main warps of R rows each, plus one halo warp.
template <typename real, int W, int R>
struct Lay {
    static constexpr int TY = W * R;
    static constexpr int NS = NSLOT;
    static constexpr int BX = Box<real>::BX;
    static constexpr int XOFF = Box<real>::XOFF;
    static constexpr int RS = (int)sizeof(real);
    // per ring slot: E boxes (TY+2 rows from j0-1), H boxes and psi_H boxes
    // (TY+1 rows from j0-1), combo and psi_E boxes (own cells, from (i0, j0))
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
    static constexpr int OFF_PE = OFF_C + CBOXP;             // 6 psi_E boxes [axis][pair]
    static constexpr int OFF_PH = OFF_PE + 6 * OBOXP;        // 6 psi_H boxes [axis][pair]
    static constexpr int SLOT = OFF_PH + 6 * HBOXP;
    static constexpr int TXB = 3 * EBOXB + 3 * HBOXB + CBOXB; // bytes per plane without psi
    static constexpr int TXPSI = 2 * OBOXB + 2 * HBOXB;       // extra bytes per CPML axis
    static constexpr int RING = NS * SLOT;
    // shared H exchange: row j0-1+w*R (Hx, Hz) per warp boundary, column i0-1 (Hy, Hz)
    static constexpr int OFF_ROW = RING;                      // [W][2][32]
    static constexpr int OFF_COL = OFF_ROW + W * 2 * FTX * RS;  // [2][TY]
    static constexpr int OFF_PROF = OFF_COL + 2 * TY * RS;    // x [4][33], y [4][TY+1]
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
// CPML state of one cell for the current plane: for each axis, whether the
// cell lies in that axis' slab, and the profile values b, c there.
template <typename real>
struct Cpml {
    bool on[3];
    real b[3], c[3];
};

// curl of component CA with its CPML terms, psi_old read from the ring
// (pin: 6 boxes [axis][pair], `pst` elements apart, at the cell's position)
// and psi_new written to global memory at offset o.  Same operation order as
// curl_psi: cur = d1 - d2; += psi(A1); -= psi(A2).
template <typename real, int CA>
__device__ __forceinline__ real curl_ring(const Cpml<real>& cp, real d1, real d2, const real* pin,
                                          int pst, real* const* pout, long long o, long long vol,
                                          bool store) {
    constexpr int A1 = (CA + 1) % 3, A2 = (CA + 2) % 3;
    constexpr int P1 = (CA > A1) ? CA - 1 : CA;
    constexpr int P2 = (CA > A2) ? CA - 1 : CA;
    real cur = d1 - d2;
    if (cp.on[A1]) {
        const real psi = cp.b[A1] * pin[(A1 * 2 + P1) * pst] + cp.c[A1] * d1;
        if (store) pout[A1][P1 * vol + o] = psi;
        cur += psi;
    }
    if (cp.on[A2]) {
        const real psi = cp.b[A2] * pin[(A2 * 2 + P2) * pst] + cp.c[A2] * d2;
        if (store) pout[A2][P2 * vol + o] = psi;
        cur -= psi;
    }
    return cur;
}

template <typename real, int W, int R>
__device__ void step_block(const InstDev<real>& I, long long local, long long n, int cur, bool dry,
                           DevState* st, unsigned char* smem) {
    using L = Lay<real, W, R>;
    constexpr int TY = L::TY, NS = L::NS;
    real* sRow = reinterpret_cast<real*>(smem + L::OFF_ROW);    // [W][Hx, Hz][32]
    real* sCol = reinterpret_cast<real*>(smem + L::OFF_COL);    // [Hy, Hz][TY]
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
    const int kend = z1;  // planes kstart..kend are read (k+1 of the last plane z1-1)

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
    // and the first MAXC_SMEM rows of the combo table
    const bool coef_smem = I.n_combos <= MAXC_SMEM;
    {
        const int t = w * FTX + tx;
        const int nthr = FTX * (W + 1);
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

    auto issue = [&](int p, int sl) {  // plane p into ring slot sl (lead thread only)
        const uint32_t bar = smem_u32(&bars[sl]);
        unsigned char* base = smem + sl * L::SLOT;
        const bool pz = have_z && (p < I.pl[2] || p >= I.nz - I.ph[2]);
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
            for (int pp = 0; pp < 2; ++pp) {
                tma_load_3d(smem_u32(base + L::OFF_PE + (a * 2 + pp) * L::OBOXP), tm + (TM_PE + a * 2 + pp) * 128,
                            i0, j0, p, bar);
                tma_load_3d(smem_u32(base + L::OFF_PH + (a * 2 + pp) * L::HBOXP),
                            tm + (TM_PH + cur * 6 + a * 2 + pp) * 128, xh, yh, p, bar);
            }
        }
    };
    if (lead)
        for (int p = kstart; p <= min(kend, kstart + NS - 1); ++p) issue(p, p - kstart);

    const real S = I.S;
    const long long vol = I.vol;
    real* const* psiHout = I.psiH[cur ^ 1];
    real* const* psiE = I.psiE;
    real* const Hx = I.F[cur ^ 1][3];
    real* const Hy = I.F[cur ^ 1][4];
    real* const Hz = I.F[cur ^ 1][5];
    real* const Ex = I.F[cur ^ 1][0];
    real* const Ey = I.F[cur ^ 1][1];
    real* const Ez = I.F[cur ^ 1][2];

    const bool main = w < W;
    const int i = i0 + tx;
    const int jb = j0 + w * R;          // first row of this warp
    const bool xin = i < I.nx;
    // halo cells of the halo warp: y-1 row (hr) and x-1 column (hc)
    const int hri = i0 + tx, hrj = j0 - 1;
    const int hci = i0 - 1, hcj = j0 + tx;
    const bool hrow = !main && hrj >= 0 && hri < I.nx;
    const bool hcol = !main && tx < TY && hci >= 0 && hcj < I.ny;
    const int xp = tx + 1;  // own column's index in the shared x profile
    const bool xon = in_slab(I, 0, i);
    const bool xon_r = in_slab(I, 0, hri), yon_r = in_slab(I, 1, hrj);
    const bool xon_c = in_slab(I, 0, hci), yon_c = in_slab(I, 1, hcj);
    const real* px = prof;                   // [4][FTX+1]
    const real* py = prof + 4 * (FTX + 1);   // [4][TY+1]
    // sources overlapping this tile's footprint (own cells and halo), one bit per source
    unsigned smask = 0;
    for (int q = 0; q < I.n_src; ++q) {
        const SrcDev<real>& sv = I.src[q];
        if (sv.lo[0] < i0 + FTX && sv.lo[0] + sv.n[0] > i0 - 1 && sv.lo[1] < j0 + TY &&
            sv.lo[1] + sv.n[1] > j0 - 1)
            smask |= 1u << q;
    }

    constexpr int EB = L::EBOXP / L::RS, HBX = L::HBOXP / L::RS, OB = L::OBOXP / L::RS;
    // shared-memory element offsets inside a ring slot, row r of this warp
    // E / H / psi_H boxes start at (i0-XOFF, j0-1); combo / psi_E boxes at (i0, j0)
    const int e_own0 = (w * R + 1) * L::BX + tx + L::XOFF;
    const int o_own0 = w * R * FTX + tx;
    const int e_row = tx + L::XOFF;                      // halo row cell (box row 0)
    const int e_col = (tx + 1) * L::BX + L::XOFF - 1;    // halo column cell

    real hx_prev[R], hy_prev[R];  // H^{n+1/2} of plane k-1 at the own cells
#pragma unroll
    for (int r = 0; r < R; ++r) hx_prev[r] = hy_prev[r] = 0;
    bool ok = true;
    int s0 = 0, s1 = 1 % NS;        // ring slots of planes k and k+1
    unsigned par0 = 0, par1 = (1 / NS) & 1;

    for (int k = kstart; k < kend; ++k) {
        const int q = k - kstart;
        const bool storing = k >= z0;
        const bool zon = have_z && (k < I.pl[2] || k >= I.nz - I.ph[2]);
        real bzi = 0, czi = 0, bzh = 0, czh = 0;
        if (zon) {
            bzi = I.prof[2][k];
            czi = I.prof[2][I.nz + k];
            bzh = I.prof[2][2 * I.nz + k];
            czh = I.prof[2][3 * I.nz + k];
        }
        unsigned pm = 0;  // sources that touch this plane (block-uniform)
        for (unsigned m = smask; m; m &= m - 1) {
            const int qq = __ffs(m) - 1;
            const SrcDev<real>& sv = I.src[qq];
            if (k >= sv.lo[2] && k < sv.lo[2] + sv.n[2]) pm |= 1u << qq;
        }
        // wait for planes k and k+1
        if (q == 0) ok &= mbar_wait(smem_u32(&bars[s0]), par0);
        ok &= mbar_wait(smem_u32(&bars[s1]), par1);
        if (!ok) abort_flag = 1;

        const real* E0 = reinterpret_cast<const real*>(smem + s0 * L::SLOT);      // E of plane k
        const real* E1 = reinterpret_cast<const real*>(smem + s1 * L::SLOT);      // E of plane k+1
        const real* H0 = reinterpret_cast<const real*>(smem + s0 * L::SLOT + L::OFF_H);
        const real* PH = reinterpret_cast<const real*>(smem + s0 * L::SLOT + L::OFF_PH);
        const real* PE = reinterpret_cast<const real*>(smem + s0 * L::SLOT + L::OFF_PE);
        const unsigned char* CBX = smem + s0 * L::SLOT + L::OFF_C;
        const long long o_plane = (long long)k * I.plane;

        real hx[R], hy[R], hz[R];
        // ---------------- H phase
        if (main) {
            const bool st_psi = storing && !dry;
#pragma unroll
            for (int r = 0; r < R; ++r) {
                const int j = jb + r;
                hx[r] = hy[r] = hz[r] = 0;
                if (!(xin && j < I.ny)) continue;
                const long long o = o_plane + (long long)j * I.px + i;
                const int eo = e_own0 + r * L::BX;
                const real* e = E0 + eo;
                const real ex = e[0], ey = e[EB], ez = e[2 * EB];
                const real ex_j = e[L::BX], ey_i = e[EB + 1], ez_i = e[2 * EB + 1], ez_j = e[2 * EB + L::BX];
                const real ex_k = E1[eo], ey_k = E1[EB + eo];
                Cpml<real> cp;
                cp.on[0] = xon;
                cp.on[1] = in_slab(I, 1, j);
                cp.on[2] = zon;
                cp.b[0] = px[2 * (FTX + 1) + xp];
                cp.c[0] = px[3 * (FTX + 1) + xp];
                cp.b[1] = py[2 * (TY + 1) + w * R + r + 1];
                cp.c[1] = py[3 * (TY + 1) + w * R + r + 1];
                cp.b[2] = bzh;
                cp.c[2] = czh;
                const real* pin = PH + eo;
                {
                    const real cv = curl_ring<real, 0>(cp, ez_j - ez, ey_k - ey, pin, HBX, psiHout, o, vol, st_psi);
                    real acc = -(S * cv);
                    if (pm) acc = apply_sources(I, SJ_HX, i, j, k, n, acc);
                    hx[r] = H0[eo] + acc;
                }
                {
                    const real cv = curl_ring<real, 1>(cp, ex_k - ex, ez_i - ez, pin, HBX, psiHout, o, vol, st_psi);
                    real acc = -(S * cv);
                    if (pm) acc = apply_sources(I, SJ_HY, i, j, k, n, acc);
                    hy[r] = H0[HBX + eo] + acc;
                }
                if (storing) {
                    const real cv = curl_ring<real, 2>(cp, ey_i - ey, ex_j - ex, pin, HBX, psiHout, o, vol, st_psi);
                    real acc = -(S * cv);
                    if (pm) acc = apply_sources(I, SJ_HZ, i, j, k, n, acc);
                    hz[r] = H0[2 * HBX + eo] + acc;
                    Hx[o] = hx[r];
                    Hy[o] = hy[r];
                    Hz[o] = hz[r];
                }
            }
            if (!storing) {
#pragma unroll
                for (int r = 0; r < R; ++r) {
                    hx_prev[r] = hx[r];
                    hy_prev[r] = hy[r];
                }
            } else if (w + 1 < W) {
                // this warp's last row is the next warp's y-1 neighbour
                sRow[(w + 1) * 2 * FTX + tx] = hx[R - 1];
                sRow[((w + 1) * 2 + 1) * FTX + tx] = hz[R - 1];
            }
        } else if (storing) {
            // halo warp: y-1 row (Hx, Hz) ...
            {
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
                    const real* pin = PH + e_row;
                    const long long o = o_plane + (long long)hrj * I.px + hri;
                    {
                        const real cv = curl_ring<real, 0>(cp, e[2 * EB + L::BX] - ez, E1[EB + e_row] - ey, pin, HBX,
                                                           psiHout, o, vol, false);
                        real acc = -(S * cv);
                        if (pm) acc = apply_sources(I, SJ_HX, hri, hrj, k, n, acc);
                        vx = H0[e_row] + acc;
                    }
                    {
                        const real cv = curl_ring<real, 2>(cp, e[EB + 1] - ey, e[L::BX] - ex, pin, HBX, psiHout, o,
                                                           vol, false);
                        real acc = -(S * cv);
                        if (pm) acc = apply_sources(I, SJ_HZ, hri, hrj, k, n, acc);
                        vz = H0[2 * HBX + e_row] + acc;
                    }
                }
                sRow[tx] = vx;
                sRow[FTX + tx] = vz;
            }
            // ... and x-1 column (Hy, Hz)
            if (tx < TY) {
                real vy = 0, vz = 0;
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
                    const real* pin = PH + e_col;
                    const long long o = o_plane + (long long)hcj * I.px + hci;
                    {
                        const real cv = curl_ring<real, 1>(cp, E1[e_col] - ex, e[2 * EB + 1] - ez, pin, HBX, psiHout,
                                                           o, vol, false);
                        real acc = -(S * cv);
                        if (pm) acc = apply_sources(I, SJ_HY, hci, hcj, k, n, acc);
                        vy = H0[HBX + e_col] + acc;
                    }
                    {
                        const real cv = curl_ring<real, 2>(cp, e[EB + 1] - ey, e[L::BX] - ex, pin, HBX, psiHout, o,
                                                           vol, false);
                        real acc = -(S * cv);
                        if (pm) acc = apply_sources(I, SJ_HZ, hci, hcj, k, n, acc);
                        vz = H0[2 * HBX + e_col] + acc;
                    }
                }
                sCol[tx] = vy;
                sCol[TY + tx] = vz;
            }
        }
        __syncthreads();

        // ---------------- E phase
        if (main && storing) {
            const bool st_in = !dry;
            const bool src_e = pm != 0;
#pragma unroll
            for (int r = 0; r < R; ++r) {
                const int j = jb + r;
                // x-1 neighbours by shuffle (lane 0 takes the halo column)
                real hy_i = __shfl_up_sync(0xffffffffu, hy[r], 1);
                real hz_i = __shfl_up_sync(0xffffffffu, hz[r], 1);
                if (tx == 0) {
                    hy_i = sCol[w * R + r];
                    hz_i = sCol[TY + w * R + r];
                }
                // y-1 neighbours from the row above (this thread, or the shared row)
                const real hx_j = r > 0 ? hx[r > 0 ? r - 1 : 0] : sRow[w * 2 * FTX + tx];
                const real hz_j = r > 0 ? hz[r > 0 ? r - 1 : 0] : sRow[(w * 2 + 1) * FTX + tx];
                if (!(xin && j < I.ny)) continue;
                const long long o = o_plane + (long long)j * I.px + i;
                const int eo = e_own0 + r * L::BX;
                const int oo = o_own0 + r * FTX;
                const int cb = CBX[oo];
                const real* cf = coef + cb * I.ncoef;
                const bool disp = (cflag[cb] & 1) != 0;
                Cpml<real> cp;
                cp.on[0] = xon;
                cp.on[1] = in_slab(I, 1, j);
                cp.on[2] = zon;
                cp.b[0] = px[xp];
                cp.c[0] = px[(FTX + 1) + xp];
                cp.b[1] = py[w * R + r + 1];
                cp.c[1] = py[(TY + 1) + w * R + r + 1];
                cp.b[2] = bzi;
                cp.c[2] = czi;
                const real* pin = PE + oo;
                const real* e = E0 + eo;
                {
                    const real cv = curl_ring<real, 0>(cp, hz[r] - hz_j, hy[r] - hy_prev[r], pin, OB, psiE, o, vol, st_in);
                    Ex[o] = e_finish_row<real, 0>(I, i, j, k, n, cf, disp, e[0], cv, st_in, src_e);
                }
                {
                    const real cv = curl_ring<real, 1>(cp, hx[r] - hx_prev[r], hz[r] - hz_i, pin, OB, psiE, o, vol, st_in);
                    Ey[o] = e_finish_row<real, 1>(I, i, j, k, n, cf, disp, e[EB], cv, st_in, src_e);
                }
                {
                    const real cv = curl_ring<real, 2>(cp, hy[r] - hy_i, hx[r] - hx_j, pin, OB, psiE, o, vol, st_in);
                    Ez[o] = e_finish_row<real, 2>(I, i, j, k, n, cf, disp, e[2 * EB], cv, st_in, src_e);
                }
            }
#pragma unroll
            for (int r = 0; r < R; ++r) {
                hx_prev[r] = hx[r];
                hy_prev[r] = hy[r];
            }
        }
        __syncthreads();
        if (abort_flag) break;
        // slot s0 is free: fetch plane k + NS into it
        if (lead && k + NS <= kend) issue(k + NS, s0);
        // advance the ring: plane k+1 is now in s0, plane k+2 in the next slot
        s0 = s1;
        par0 = par1;
        if (++s1 == NS) s1 = 0;
        par1 = (unsigned)(((q + 2) / NS) & 1);
    }
    if (abort_flag) {
        if (lead) {
            st->status = SJ_E_TIMEOUT;
            // bounded wait for every copy this block may still have in flight
            for (int qq = 0; qq < NS; ++qq) mbar_wait(smem_u32(&bars[qq]), 0), mbar_wait(smem_u32(&bars[qq]), 1);
        }
        __syncthreads();
    }
}

template <typename real, int W, int R>
__global__ void __launch_bounds__(FTX * (W + 1))
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
        step_block<real, W, R>(sI, lb - pre[ii], n, cur, fl.dry != 0, st, smem);
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

template <typename real, int W, int R>
static cudaError_t launch_wr(const InstDev<real>* d, int n_inst, DevState* st, const FusedLaunch& fl,
                             cudaStream_t s) {
    using L = Lay<real, W, R>;
    const int bytes = L::BYTES > 2 * MAXF_FUSED * 16 ? L::BYTES : 2 * MAXF_FUSED * 16;
    if (bytes > FUSED_MAX_SMEM) return cudaErrorInvalidConfiguration;
    static bool attr = false;
    if (!attr) {
        cudaError_t e = cudaFuncSetAttribute(k_fused<real, W, R>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
        if (e != cudaSuccess) return e;
        attr = true;
    }
    const long long blocks = fl.n_items + fl.n_probe_blocks;
    k_fused<real, W, R><<<(unsigned)blocks, dim3(FTX, W + 1), bytes, s>>>(d, n_inst, st, fl);
    return cudaGetLastError();
}

// Supported tilings: (tile rows, rows per thread) -> W = tile_y / rows main warps.
#define SJ_FUSED_TILINGS(X) X(4, 1) X(8, 1) X(16, 1) X(8, 2) X(16, 2)

template <typename real>
cudaError_t launch_fused_step(const InstDev<real>* d_insts, int n_inst, DevState* st,
                              const FusedLaunch& fl, cudaStream_t s) {
#define SJ_CASE(TYV, RV) \
    if (fl.ty == TYV && fl.rows == RV) return launch_wr<real, TYV / RV, RV>(d_insts, n_inst, st, fl, s);
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
int fused_block_threads(int ty, int rows) { return FTX * (ty / rows + 1); }

template <typename real>
int fused_smem_bytes(int ty, int rows) {
#define SJ_CASE(TYV, RV) \
    if (ty == TYV && rows == RV) return Lay<real, TYV / RV, RV>::BYTES;
    SJ_FUSED_TILINGS(SJ_CASE)
#undef SJ_CASE
    return -1;
}
template int fused_smem_bytes<float>(int, int);
template int fused_smem_bytes<double>(int, int);
int fused_tensor_maps() { return TM_COUNT; }

template cudaError_t launch_fused_step<double>(const InstDev<double>*, int, DevState*, const FusedLaunch&,
                                               cudaStream_t);
template cudaError_t launch_fused_step<float>(const InstDev<float>*, int, DevState*, const FusedLaunch&,
                                              cudaStream_t);
}  // namespace sj
