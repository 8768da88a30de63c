// Dust-attenuated FUV field G0 = sum_star L exp(-tau_FUV) / r^2.  Follows
// nebula3d.py:320-352 (cast_fuv: per-ray dust optical depth binned on a coarse spherical
// grid att[r, u, phi]) and nebula3d.py:355-388 (apply_fuv: trilinear att / r^2 per cell),
// as driven by sim.py:949-985 (fuv_field, fp16 store of G0).
//
// GB300 design: cast_fuv marches a ray with a group of G lanes, the optical depth being an
// inclusive group scan over a Kahan-compensated carry; a lane that crosses into new radial
// bins writes them, and a ray stops once its optical depth passes 120 (exp(-tau) is 0.0f from
// there on: its remaining bins are written as 0).  Density and ionized fraction are sampled at the same corners, so they
// are first packed as (rho, xi) pairs into free scratch: one 8-byte gather per corner.  All rays of all active stars are one launch, into one attenuation grid
// per star laid out [star][u][phi][r] (r fastest: a ray's bins are contiguous).  Each entry is
// the pair (att(r), att(min(r + 1, nr - 1))) as one float2 (the ray writes each bin into its own
// pair and its lower neighbour's), so a trilinear sample of apply_fuv is four 8-byte gathers
// instead of eight 4-byte ones; values and arithmetic are those of the plain table
// (NB_TUNE_FUV_PAIRS = 0), bit for bit.  apply_fuv accumulates every active star for a cell in
// one register, in the reference's star order (so the float32 sum is the reference's), and
// stores G0 once as fp16.
#include "nb_rayutil.cuh"

namespace {

__global__ void __launch_bounds__(256) pack_rx_kernel(const float* __restrict__ rho, const float* __restrict__ xi,
                                                      float2* __restrict__ rx, long long n) {
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n; q += (long long)gridDim.x * blockDim.x)
        rx[q] = make_float2(rho[q], xi[q]);
}

template <int G, bool REF_LAYOUT, bool PAIRS>
__global__ void __launch_bounds__(256, 5) cast_fuv_kernel(const NbConst* __restrict__ c, const NbStarW* __restrict__ sw,
                                                       const float4* __restrict__ dirs,
                                                       const float2* __restrict__ rx,
                                                       float* __restrict__ att, int nstars,
                                                       const float* star_override, float tau_cut) {
    const int nr = c->fnr, nu = c->fnu, nphi = c->fnphi, nray = nu * nphi;
    const long long gid = (blockIdx.x * (long long)blockDim.x + threadIdx.x) / G;
    const int lane = threadIdx.x % G;
    const unsigned gmask = G == 32 ? 0xffffffffu : (((1u << G) - 1u) << ((threadIdx.x & 31) / G * G));
    if (gid >= (long long)nray * nstars) return;
    // below 2^32 (fnu * fnphi * nstars; nb_create checks it): 32-bit division
    const int s = (int)((unsigned)gid / (unsigned)nray), ray = (int)((unsigned)gid - (unsigned)s * (unsigned)nray);
    float sx, sy, sz;
    if (star_override) {
        sx = star_override[0]; sy = star_override[1]; sz = star_override[2];
    } else {
        const NbStarW w = sw[s];
        if (!w.active) return;
        sx = w.w.x; sy = w.w.y; sz = w.w.z;
    }
    const int iu = ray / nphi, ip = ray % nphi;
    // bin b of this ray: the reference layout [b][iu][ip], or the instance's [star][u][phi][b] (a ray's
    // bins contiguous; a u-fastest layout makes the apply's gathers contiguous but scatters these writes,
    // a net loss measured at 256^3)
    auto put = [&](int b, float v) {
        if (REF_LAYOUT) {
            att[((long long)b * nu + iu) * nphi + ip] = v;
        } else if (!PAIRS) {
            att[((long long)s * nray + ray) * nr + b] = v;
        } else {                                 // bin b is pair b's .x and pair b-1's .y
            float* p = att + 2 * (((long long)s * nray + ray) * nr + b);
            p[0] = v;
            if (b > 0) p[-1] = v;
            if (b == nr - 1) p[1] = v;
        }
    };
    const int nx = c->nx, ny = c->ny, nz = c->nz;
    const float dx = c->dx, inv_dx = c->inv_dx, dr = c->dr_f, binr = c->binr_f, kappa = c->kappa_f;
    const bool pow2 = c->dx_pow2 != 0;
    const float4 d = dirs[ray];
    float t0, t1;
    nb_box_range(sx, sy, sz, d.x, d.y, d.z, c->bmax, t0, t1);
    const int n0 = trunc_i(t0 / dr);
    const int n1 = min(c->nsteps, trunc_i(t1 / dr) + 2);
    float hi = 0.0f, comp = 0.0f;      // Kahan-compensated optical depth carried between segments
    int ib = 0;                        // first bin not yet written
    bool stopped = false;
    for (int base = n0; base < n1; base += G) {
        const int n = base + lane;
        const bool valid = n < n1;
        const float r = ((float)n + 0.5f) * dr;
        float dtau = 0.0f;
        int nb = ib;
        if (valid) {
            const float qx = sx + d.x * r, qy = sy + d.y * r, qz = sz + d.z * r;
            const float2 nx_i = sample_n2(rx, nx, ny, nz, qx, qy, qz, dx, inv_dx, pow2);   // (n_tot, x_i)
            dtau = kappa * nx_i.x * (1.0f - 0.92f * nx_i.y) * dr;
            nb = trunc_i(r / binr);
        }
        float incl = dtau;
#pragma unroll
        for (int o = 1; o < G; o <<= 1) {
            const float v = __shfl_up_sync(gmask, incl, o, G);
            if (lane >= o) incl = incl + v;
        }
        const float tau = hi + (incl - comp);
        // bins [prev, min(nb, nr)) take exp(-tau) of this sample (nb never decreases along a ray)
        int prev = __shfl_up_sync(gmask, nb, 1, G);
        if (lane == 0) prev = ib;
        const bool stop = valid && nb >= nr;
        // Past tau_cut (> 0) exp(-tau) is 0.0f (exp(-120) ~ 8e-53 lies far below the least float
        // denormal) and stays 0 along the ray (dtau >= 0): the bins from here on are all 0.
        const bool dark = tau_cut > 0.0f && valid && tau > tau_cut;
        const unsigned bal = __ballot_sync(gmask, stop || dark);
        const unsigned mine = G == 32 ? bal : (bal >> ((threadIdx.x & 31) / G * G)) & ((1u << G) - 1u);
        const int first_stop = mine ? __ffs(mine) - 1 : G;
        if (valid && lane <= first_stop && nb > prev) {
            const float v = expf(-tau);
            const int e = min(nb, nr);
            for (int b = prev; b < e; ++b) put(b, v);
        }
        if (mine) {                              // a lane ran out of bins or into the dark
            const int e_first = __shfl_sync(gmask, min(nb, nr), first_stop, G);
            for (int b = e_first + lane; b < nr; b += G) put(b, 0.0f);
            stopped = true;
            break;
        }
        const int last = min(G, n1 - base) - 1;
        ib = __shfl_sync(gmask, nb, last, G);
        const float total = __shfl_sync(gmask, incl, G - 1, G);
        const float y = total - comp;
        const float tsum = hi + y;
        comp = (tsum - hi) - y;
        hi = tsum;
    }
    if (!stopped) {
        const float v = expf(-(hi - comp));
        for (int b = ib + lane; b < nr; b += G) put(b, v);
    }
}

template <bool HALF, bool PAIRS>
__global__ void __launch_bounds__(256, 6) apply_fuv_kernel(const NbConst* __restrict__ c, const NbStarW* __restrict__ sw,
                                                        const float* __restrict__ att, int nstars,
                                                        void* __restrict__ g0) {
    __shared__ float4 st[NB_MAX_STARS];
    __shared__ float lum[NB_MAX_STARS];
    __shared__ int act[NB_MAX_STARS];
    __shared__ float4 rowtab[8][NB_ROW_STARS];
    for (int s = threadIdx.y * blockDim.x + threadIdx.x; s < nstars; s += blockDim.x * blockDim.y) {
        st[s] = sw[s].w;
        lum[s] = sw[s].lum_f;
        act[s] = sw[s].active;
    }
    __syncthreads();
    const int nx = c->nx, ny = c->ny, nz = c->nz, nr = c->fnr, nu = c->fnu, nphi = c->fnphi;
    const float dx = c->dx, binr = c->binr_f;
    const float two_pi = 2.0f * pi_f();
    const int C_plane_on = c->plane_on;
    const float* C_plane_g0 = c->plane_g0;
    const RowWalk w(nx, ny, nz);
    if (!w.valid) return;
    const float px = ((float)w.i + 0.5f) * dx, py = ((float)w.j + 0.5f) * dx;
    // per-row azimuth constants (star_row_table): the same values the per-cell form computes
    float4* tab = nstars <= NB_ROW_STARS ? rowtab[threadIdx.y] : nullptr;
    if (tab) star_row_table(st, act, nstars, px, py, nphi, 1, tab);
    for (int k = w.k0; k < nz; k += 32) {
        const long long q = w.base + k;
        const float pz = ((float)k + 0.5f) * dx;
        float g = 0.0f;
        constexpr int SG = 2;                    // stars whose gathers are in flight together
        for (int s0 = 0; s0 < nstars; s0 += SG) {
          float term[SG];
          bool on[SG];
#pragma unroll
          for (int e = 0; e < SG; ++e) {
            const int s = s0 + e;
            on[e] = s < nstars && act[s];
            term[e] = 0.0f;
            if (!on[e]) continue;
            const float4 sp = st[s];
            const float rz = pz - sp.z;
            float r, tp;
            int pw[2];
            if (tab) {
                const float4 tb = tab[s];
                r = fmaxq(sqrtf(tb.x + rz * rz), 1e-6f);                          // (rx^2 + ry^2) + rz^2
                tp = tb.y;
                pw[0] = __float_as_int(tb.z);
                pw[1] = __float_as_int(tb.w);
            } else {
                const float rx = px - sp.x, ry = py - sp.y;
                r = fmaxq(sqrtf((rx * rx + ry * ry) + rz * rz), 1e-6f);             // 0 + x*x == x*x
                float phi = atan2f(ry, rx);
                if (phi < 0.0f) phi = phi + two_pi;
                const float fp = phi / two_pi * (float)nphi - 0.5f;
                const int ip = (int)floorf(fp);
                tp = fp - (float)ip;
                pw[0] = wrap_index(ip, nphi);
                pw[1] = wrap_index(ip + 1, nphi);
            }
            const float u = rz / r;
            const float fr = r / binr - 0.5f;
            const float fu = (u + 1.0f) * 0.5f * (float)nu - 0.5f;
            const int ir = (int)floorf(fr), iu = (int)floorf(fu);
            const float tr = fr - (float)ir, tu = fu - (float)iu;
            const long long tab0 = (long long)s * nu * nphi * nr;
            float v[2][2][2];                    // [r corner][u corner][phi corner]
            if (PAIRS) {
                // pair rc = (att(rc), att(min(rc + 1, nr - 1))): the two r corners, except at ir = -1,
                // where both clamp to r = 0 (the pair's .x)
                const float2* ap = reinterpret_cast<const float2*>(att) + tab0;
                const int rc = iclampd(ir, 0, nr - 1);
#pragma unroll
                for (int bb = 0; bb < 2; ++bb)
#pragma unroll
                    for (int cc = 0; cc < 2; ++cc) {
                        const int uu = iclampd(iu + bb, 0, nu - 1);
                        const float2 pr = __ldg(ap + ((uu * nphi + pw[cc]) * nr + rc));      // < 2^31 per star
                        v[0][bb][cc] = pr.x;
                        v[1][bb][cc] = ir < 0 ? pr.x : pr.y;
                    }
            } else {
                const float* as = att + tab0;
#pragma unroll
                for (int aa = 0; aa < 2; ++aa)
#pragma unroll
                    for (int bb = 0; bb < 2; ++bb)
#pragma unroll
                        for (int cc = 0; cc < 2; ++cc) {
                            const int rr = iclampd(ir + aa, 0, nr - 1);
                            const int uu = iclampd(iu + bb, 0, nu - 1);
                            v[aa][bb][cc] = __ldg(as + ((uu * nphi + pw[cc]) * nr + rr));   // < 2^31 per star
                        }
            }
            float acc = 0.0f;
#pragma unroll
            for (int aa = 0; aa < 2; ++aa)
#pragma unroll
                for (int bb = 0; bb < 2; ++bb)
#pragma unroll
                    for (int cc = 0; cc < 2; ++cc) {
                        const float wgt = (aa == 0 ? 1.0f - tr : tr) * (bb == 0 ? 1.0f - tu : tu) * (cc == 0 ? 1.0f - tp : tp);
                        acc = acc + wgt * v[aa][bb][cc];
                    }
            const float r2 = fmaxq(r * r, 0.0004f);
            term[e] = lum[s] * acc / r2;
          }
#pragma unroll
          for (int e = 0; e < SG; ++e)
            if (on[e]) g = g + term[e];                 // the reference's star order
        }
        if (C_plane_on) g = g + __ldg(C_plane_g0 + q);      // the -x plane source, after the stars
        if (HALF)
            reinterpret_cast<__half*>(g0)[q] = __float2half_rn(g);
        else
            reinterpret_cast<float*>(g0)[q] = g;
    }
}

// FUV of the -x plane source (no reference counterpart): per column, the dust optical depth
// of nebula3d.py:343 summed along +x to each cell centre; G0 term = L exp(-tau).
__global__ void __launch_bounds__(256) plane_fuv_kernel(const NbConst* __restrict__ c, const float* __restrict__ rho,
                                                        const float* __restrict__ xi, float* __restrict__ g) {
    const int nx = c->nx, ny = c->ny, nz = c->nz;
    const int col = blockIdx.x * blockDim.x + threadIdx.x;
    if (col >= ny * nz) return;
    const float kappa = c->kappa_f, dx = c->dx, lum = c->plane_lum_f;
    const long long plane = (long long)ny * nz;
    float tau = 0.0f;
    for (int i = 0; i < nx; ++i) {
        const long long q = i * plane + col;
        const float dtau = kappa * __ldg(rho + q) * (1.0f - 0.92f * __ldg(xi + q)) * dx;
        g[q] = lum * expf(-(tau + 0.5f * dtau));
        tau = tau + dtau;
    }
}

}  // namespace

cudaError_t nb_launch_plane_fuv(const NbConst* c, const float* rho, const float* xi, float* g, int ny, int nz,
                                cudaStream_t s) {
    const int cols = ny * nz;
    plane_fuv_kernel<<<(cols + 255) / 256, 256, 0, s>>>(c, rho, xi, g);
    return cudaGetLastError();
}

cudaError_t nb_launch_cast_fuv(const NbConst* c, const NbStarW* sw, const float4* dirs, const float* rho,
                               const float* xi, float* att, int nstars, int group, const float* star_override,
                               int ref_layout, cudaStream_t s, int fnu, int fnphi, void* rx_scratch, long long ncell,
                               float tau_cut, int pairs) {
    float2* rx = static_cast<float2*>(rx_scratch);
    {
        const long long b = (ncell + 255) / 256;
        pack_rx_kernel<<<(int)(b < 152LL * 16 ? (b < 1 ? 1 : b) : 152LL * 16), 256, 0, s>>>(rho, xi, rx, ncell);
    }
    const long long threads = (long long)fnu * fnphi * nstars * group;
    const int blocks = (int)((threads + 255) / 256);
#define NB_FUV_LAUNCH(G, R, PR) \
    cast_fuv_kernel<G, R, PR><<<blocks, 256, 0, s>>>(c, sw, dirs, rx, att, nstars, star_override, tau_cut)
    if (ref_layout) {
        NB_FUV_LAUNCH(32, true, false);
    } else if (pairs) {
        switch (group) {
            case 8: NB_FUV_LAUNCH(8, false, true); break;
            case 16: NB_FUV_LAUNCH(16, false, true); break;
            default: NB_FUV_LAUNCH(32, false, true); break;
        }
    } else {
        switch (group) {
            case 8: NB_FUV_LAUNCH(8, false, false); break;
            case 16: NB_FUV_LAUNCH(16, false, false); break;
            default: NB_FUV_LAUNCH(32, false, false); break;
        }
    }
#undef NB_FUV_LAUNCH
    return cudaGetLastError();
}

cudaError_t nb_launch_apply_fuv(const NbConst* c, const NbStarW* sw, const float* att, int nstars, void* g0,
                                cudaStream_t s, int nx, int ny, int half, int pairs) {
    const int blocks = rowwalk_blocks(nx, ny);
    if (half && pairs)
        apply_fuv_kernel<true, true><<<blocks, dim3(32, 8), 0, s>>>(c, sw, att, nstars, g0);
    else if (half)
        apply_fuv_kernel<true, false><<<blocks, dim3(32, 8), 0, s>>>(c, sw, att, nstars, g0);
    else if (pairs)
        apply_fuv_kernel<false, true><<<blocks, dim3(32, 8), 0, s>>>(c, sw, att, nstars, g0);
    else
        apply_fuv_kernel<false, false><<<blocks, dim3(32, 8), 0, s>>>(c, sw, att, nstars, g0);
    return cudaGetLastError();
}
