// Stromgren ionization: per-star ray casting of the recombination column, the front
// apply (max-merge of xi, min-merge of the signed front distance) and the 7-point
// smoothing of xi.  Follows nebula3d.py:195-315 (sample_n, box_range, cast_rays, rf_at,
// apply_front, smooth_xi) as driven by sim.py:927-947 (ionize).
//
// GB300 design:
//  * cast_rays: a group of G lanes (G = 32: one warp) marches one ray, G consecutive samples
//    at a time; the recombination column sum(n^2 r^2 dr) is an inclusive group scan on top
//    of a Kahan-compensated carry, and the first sample whose column passes Q is found with
//    one ballot.  All rays of all active stars are one launch.
//  * apply_front: every active star merges into one register pair per cell (max / min are
//    exact and order-free, so one pass over the grid equals the reference's S passes); the
//    float32 front distance is rounded once to the fp16 dfront (sim.py:980-985, 511-514).
//  * smooth_xi writes the final xi and reduces the CFL max speed of the step from it
//    (nebula3d.py:154-162), so an ionizing step needs no separate max-speed pass.
#include "nb_rayutil.cuh"

namespace {

// Ray directions of nebula3d.py:253-256 / 329-332 in float32; cos/sin of the float32 angle
// are evaluated in FP64 and rounded (the correctly rounded float32 value in all but
// vanishingly rare double-rounding cases).  Computed once per ray grid.
__global__ void ray_dirs_kernel(int nu, int nphi, float4* __restrict__ dirs) {
    const int id = blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= nu * nphi) return;
    const int iu = id / nphi, ip = id % nphi;
    const float u = -1.0f + ((float)iu + 0.5f) * 2.0f / (float)nu;
    const float s = sqrtf(fmaxr(1.0f - u * u, 0.0f));
    const float phi = ((float)ip + 0.5f) * 2.0f * pi_f() / (float)nphi;
    const float cph = (float)cos((double)phi), sph = (float)sin((double)phi);
    dirs[id] = make_float4(s * cph, s * sph, u, 0.0f);
}

// nebula3d.py:247-270 cast_rays, G lanes per ray.
template <int G>
__global__ void __launch_bounds__(256) cast_rays_kernel(const NbConst* __restrict__ c, const NbStarW* __restrict__ sw,
                                                        const float4* __restrict__ dirs,
                                                        const float* __restrict__ rho, float* __restrict__ rfront,
                                                        int nstars, const float* star_override, float q_override) {
    const int nu = c->nu, nphi = c->nphi, nray = nu * nphi;
    const long long gid = (blockIdx.x * (long long)blockDim.x + threadIdx.x) / G;
    const int lane = threadIdx.x % G;
    const unsigned gmask = G == 32 ? 0xffffffffu : (((1u << G) - 1u) << ((threadIdx.x & 31) / G * G));
    if (gid >= (long long)nray * nstars) return;
    const int s = (int)(gid / nray), ray = (int)(gid % nray);
    float sx, sy, sz, Q;
    if (star_override) {
        sx = star_override[0]; sy = star_override[1]; sz = star_override[2]; Q = q_override;
    } else {
        const NbStarW w = sw[s];
        if (!w.active) return;
        sx = w.w.x; sy = w.w.y; sz = w.w.z; Q = w.q_f;
    }
    const int nx = c->nx, ny = c->ny, nz = c->nz;
    const float dx = c->dx, inv_dx = c->inv_dx, dr = c->dr_f;
    const bool pow2 = c->dx_pow2 != 0;
    const float4 d = dirs[ray];
    float t0, t1;
    nb_box_range(sx, sy, sz, d.x, d.y, d.z, c->bmax, t0, t1);
    const int n0 = trunc_i(t0 / dr);
    const int n1 = min(c->nsteps, trunc_i(t1 / dr) + 2);
    float hi = 0.0f, comp = 0.0f;          // Kahan-compensated column carried between segments
    float rf = c->diag_f;
    for (int base = n0; base < n1; base += G) {
        const int n = base + lane;
        const bool valid = n < n1;
        const float r = ((float)n + 0.5f) * dr;
        float inc = 0.0f;
        if (valid) {
            const float nv = sample_n(rho, nx, ny, nz, sx + d.x * r, sy + d.y * r, sz + d.z * r, dx, inv_dx, pow2);
            inc = nv * nv * r * r * dr;
        }
        float incl = inc;
#pragma unroll
        for (int o = 1; o < G; o <<= 1) {
            const float v = __shfl_up_sync(gmask, incl, o, G);
            if (lane >= o) incl = incl + v;
        }
        float excl = __shfl_up_sync(gmask, incl, 1, G);
        if (lane == 0) excl = 0.0f;
        const float col = hi + (excl - comp);
        const bool cross = valid && (col + inc > Q);
        const unsigned bal = __ballot_sync(gmask, cross);
        const unsigned mine = G == 32 ? bal : (bal >> ((threadIdx.x & 31) / G * G)) & ((1u << G) - 1u);
        if (mine) {
            const int f = __ffs(mine) - 1;
            const float rfl = r - 0.5f * dr + dr * (Q - col) / fmaxr(inc, 1e-20f);
            rf = __shfl_sync(gmask, rfl, f, G);
            break;
        }
        const float total = __shfl_sync(gmask, incl, G - 1, G);
        const float y = total - comp;
        const float tsum = hi + y;
        comp = (tsum - hi) - y;
        hi = tsum;
    }
    if (lane == 0) rfront[(long long)s * nray + ray] = rf;
}

// nebula3d.py:273-307 rf_at + apply_front, fused over the active stars, with the fp16
// store of the front distance (sim.py:942, 980-985).
template <bool HALF>
__global__ void __launch_bounds__(256) apply_front_kernel(const NbConst* __restrict__ c,
                                                          const NbStarW* __restrict__ sw,
                                                          const float* __restrict__ rfront, int nstars,
                                                          float* __restrict__ xi_raw, void* __restrict__ dfront,
                                                          unsigned* smax_reset) {
    __shared__ float4 st[NB_MAX_STARS];
    __shared__ int act[NB_MAX_STARS];
    const int tlin = threadIdx.y * blockDim.x + threadIdx.x;
    for (int s = tlin; s < nstars; s += blockDim.x * blockDim.y) {
        st[s] = sw[s].w;
        act[s] = sw[s].active;
    }
    __syncthreads();
    if (smax_reset && blockIdx.x == 0 && tlin == 0) *smax_reset = 0u;
    const int nx = c->nx, ny = c->ny, nz = c->nz, nu = c->nu, nphi = c->nphi;
    const float dx = c->dx, width = c->width;
    const float two_pi = 2.0f * pi_f();
    const RowWalk w(nx, ny, nz);
    if (!w.valid) return;
    const float px = ((float)w.i + 0.5f) * dx, py = ((float)w.j + 0.5f) * dx;
    for (int k = w.k0; k < nz; k += 32) {
        const long long q = w.base + k;
        const float pz = ((float)k + 0.5f) * dx;
        float xi = 0.0f, df = 1e3f;
        for (int s = 0; s < nstars; ++s) {
            if (!act[s]) continue;
            const float4 sp = st[s];
            const float rx = px - sp.x, ry = py - sp.y, rz = pz - sp.z;
            const float r = fmaxr(sqrtf((rx * rx + ry * ry) + rz * rz), 1e-6f);     // 0 + x*x == x*x
            const float u = rz / r;
            float phi = atan2f(ry, rx);
            if (phi < 0.0f) phi = phi + two_pi;
            const float fu = (u + 1.0f) * 0.5f * (float)nu - 0.5f;
            const float fp = phi / two_pi * (float)nphi - 0.5f;
            const int iu = (int)floorf(fu), ip = (int)floorf(fp);
            const float tu = fu - (float)iu, tp = fp - (float)ip;
            const float* rfs = rfront + (long long)s * nu * nphi;
            const int u0 = iclampd(iu, 0, nu - 1), u1 = iclampd(iu + 1, 0, nu - 1);
            const int p0 = wrap_index(ip, nphi), p1 = wrap_index(ip + 1, nphi);
            const float ra = __ldg(rfs + u0 * nphi + p0) * (1.0f - tp) + __ldg(rfs + u0 * nphi + p1) * tp;
            const float rb = __ldg(rfs + u1 * nphi + p0) * (1.0f - tp) + __ldg(rfs + u1 * nphi + p1) * tp;
            const float rf = ra * (1.0f - tu) + rb * tu;
            const float val = fminr(fmaxr(0.0f, (rf - r) / width + 0.5f), 1.0f);
            if (val > xi) xi = val;
            df = fminr(df, r - rf);
        }
        xi_raw[q] = xi;
        if (HALF)
            reinterpret_cast<__half*>(dfront)[q] = __float2half_rn(df);
        else
            reinterpret_cast<float*>(dfront)[q] = df;
    }
}

// nebula3d.py:310-315 smooth_xi (+ sim.py:941 copy back), then the CFL max speed
// (nebula3d.py:154-162) of the state with the new xi.
__global__ void __launch_bounds__(256) smooth_kernel(const NbConst* __restrict__ c, const float* __restrict__ src,
                                                     float* __restrict__ xi, const float* __restrict__ rho,
                                                     const float* __restrict__ mx, const float* __restrict__ my,
                                                     const float* __restrict__ mz, unsigned* smax_bits) {
    const int nx = c->nx, ny = c->ny, nz = c->nz;
    const float cn2 = c->cn2, ci2 = c->ci2;
    float m = 0.0f;
    const RowWalk w(nx, ny, nz);
    if (w.valid) {
        const long long sj = nz, si = (long long)ny * nz;
        const long long dxm = w.i > 0 ? si : 0, dxp = w.i < nx - 1 ? si : 0;
        const long long dym = w.j > 0 ? sj : 0, dyp = w.j < ny - 1 ? sj : 0;
        for (int k = w.k0; k < nz; k += 32) {
            const long long q = w.base + k;
            const float xm = __ldg(src + q - dxm), xp = __ldg(src + q + dxp);
            const float ym = __ldg(src + q - dym), yp = __ldg(src + q + dyp);
            const float zm = __ldg(src + q - (k > 0 ? 1 : 0)), zp = __ldg(src + q + (k < nz - 1 ? 1 : 0));
            const float mm = (xm + xp + ym + yp + zm + zp) / 6.0f;
            const float x = 0.5f * __ldg(src + q) + 0.5f * mm;
            xi[q] = x;
            if (smax_bits) {
                const float r = rho[q];
                const float v = fabsf(mx[q] / r) + fabsf(my[q] / r) + fabsf(mz[q] / r) + sqrtf(cn2 + x * (ci2 - cn2));
                m = fmaxr(v, m);
            }
        }
    }
    if (!smax_bits) return;
    for (int o = 16; o > 0; o >>= 1) m = fmaxr(m, __shfl_xor_sync(0xffffffffu, m, o));
    __shared__ float red[32];
    if (threadIdx.x == 0) red[threadIdx.y] = m;
    __syncthreads();
    if (threadIdx.x == 0 && threadIdx.y == 0) {
        float b = 0.0f;
        for (int w = 0; w < (int)blockDim.y; ++w) b = fmaxr(b, red[w]);
        atomicMax(smax_bits, __float_as_uint(b));
    }
}

}  // namespace

cudaError_t nb_launch_ray_dirs(int nu, int nphi, float4* dirs, cudaStream_t s) {
    const int n = nu * nphi;
    ray_dirs_kernel<<<(n + 255) / 256, 256, 0, s>>>(nu, nphi, dirs);
    return cudaGetLastError();
}

cudaError_t nb_launch_cast_rays(const NbConst* c, const NbStarW* sw, const float4* dirs, const float* rho,
                                float* rfront, int nstars, int group, const float* star_override, float q_override,
                                cudaStream_t s, int nu, int nphi) {
    const long long threads = (long long)nu * nphi * nstars * group;
    const int blocks = (int)((threads + 255) / 256);
    switch (group) {
        case 4: cast_rays_kernel<4><<<blocks, 256, 0, s>>>(c, sw, dirs, rho, rfront, nstars, star_override, q_override); break;
        case 8: cast_rays_kernel<8><<<blocks, 256, 0, s>>>(c, sw, dirs, rho, rfront, nstars, star_override, q_override); break;
        case 16: cast_rays_kernel<16><<<blocks, 256, 0, s>>>(c, sw, dirs, rho, rfront, nstars, star_override, q_override); break;
        default: cast_rays_kernel<32><<<blocks, 256, 0, s>>>(c, sw, dirs, rho, rfront, nstars, star_override, q_override); break;
    }
    return cudaGetLastError();
}

cudaError_t nb_launch_apply_front(const NbConst* c, const NbStarW* sw, const float* rfront, int nstars,
                                  float* xi_raw, void* dfront, unsigned* smax_reset, cudaStream_t s, int nx, int ny,
                                  int half) {
    const dim3 blk(32, 8);
    const int blocks = rowwalk_blocks(nx, ny);
    if (half)
        apply_front_kernel<true><<<blocks, blk, 0, s>>>(c, sw, rfront, nstars, xi_raw, dfront, smax_reset);
    else
        apply_front_kernel<false><<<blocks, blk, 0, s>>>(c, sw, rfront, nstars, xi_raw, dfront, smax_reset);
    return cudaGetLastError();
}

cudaError_t nb_launch_smooth(const NbConst* c, const float* xi_raw, float* xi, const float* rho, const float* mx,
                             const float* my, const float* mz, unsigned* smax_bits, cudaStream_t s, int nx, int ny) {
    smooth_kernel<<<rowwalk_blocks(nx, ny), dim3(32, 8), 0, s>>>(c, xi_raw, xi, rho, mx, my, mz, smax_bits);
    return cudaGetLastError();
}
