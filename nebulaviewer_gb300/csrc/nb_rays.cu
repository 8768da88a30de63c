// Stromgren ionization: per-star ray casting of the recombination column, the front
// apply (max-merge of xi, min-merge of the signed front distance) and the 7-point
// smoothing of xi.  Follows nebula3d.py:195-315 (sample_n, box_range, cast_rays, rf_at,
// apply_front, smooth_xi) as driven by sim.py:927-947 (ionize).
//
// GB300 design:
//  * cast_rays: a group of G lanes (1 to 32; 1 by default) marches one ray, G consecutive
//    samples at a time; the recombination column sum(n^2 r^2 dr) is added to a Kahan-compensated
//    carry (G > 1: an inclusive group scan; two lanes take it from one exchange; one lane needs
//    none, which made it the fastest shape once the shuffles' latency led the stalls), and the
//    first sample whose column passes Q is found with one ballot.  The march is warp-uniform: a
//    warp's groups loop together until all are done, and the trilinear sampler has no branches,
//    so the lanes never diverge (divergent exits had made branch resolution the leading stall).
//    All rays of all active stars are one launch.
//  * The front table holds, per (star, phi, u), the pair (rf(u), rf(min(u + 1, nu - 1))) as one
//    float2 (cast_rays writes each front into its own pair and its lower neighbour's), so the
//    bilinear lookup of apply_front is two 8-byte gathers instead of four 4-byte ones; the values
//    and the arithmetic are those of the plain table (NB_TUNE_FRONT_PAIRS = 0), bit for bit.
//  * apply_front: one pass over the grid merges the active stars, in star order, into one
//    register pair per cell (the reference makes S passes).  With up to 32 stars, each star's
//    front-radius range (front_bounds_kernel) lets a 32-cell row segment leave out the stars that
//    cannot change its xi or front distance (the same bits).  The float32 front distance is
//    rounded once to the fp16 dfront (sim.py:980-985, 511-514).
//  * smooth_xi writes the final xi and reduces the CFL max speed of the step from it
//    (nebula3d.py:154-162), so an ionizing step needs no separate max-speed pass.
#include <cstring>

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

// nebula3d.py:247-270 cast_rays: ray `ray` of star (sx, sy, sz, Q), G lanes per ray.  `out` is where
// the front radius goes (a float pointer, 4-byte aligned) with two flags in its low bits: bit 0 also
// writes out[-1] and bit 1 out[1] (the pair layout's neighbour copies, front_slot); one 64-bit
// value stays live across the march, as a plain pointer would.
template <int G>
__device__ __forceinline__ void cast_ray(const NbConst& C, const float4* __restrict__ dirs,
                                         const float* __restrict__ rho, uintptr_t out, int ray, float sx, float sy,
                                         float sz, float Q, int lane, unsigned gmask, bool live) {
    // Warp-uniform march: every lane of the warp runs the loop until all of its groups are done
    // (`live` false: the group has no ray; `ray` is then any valid index), a finished group's lanes
    // only carry predicated-off values, so the warp never diverges inside the loop.
    const int nx = C.nx, ny = C.ny, nz = C.nz;
    const float dx = C.dx, inv_dx = C.inv_dx, dr = C.dr_f;
    const bool pow2 = C.dx_pow2 != 0;
    const float4 d = dirs[ray];
    float t0, t1;
    nb_box_range(sx, sy, sz, d.x, d.y, d.z, C.bmax, t0, t1);
    const int n0 = trunc_i(t0 / dr);
    const int n1 = min(C.nsteps, trunc_i(t1 / dr) + 2);
    float hi = 0.0f, comp = 0.0f;          // Kahan-compensated column carried between segments
    float rf = C.diag_f;
    bool done = !live || n0 >= n1;
    for (int base = n0;; base += G) {
        if (__all_sync(0xffffffffu, done)) break;
        const int n = base + lane;
        const bool valid = !done && n < n1;
        const float r = ((float)n + 0.5f) * dr;
        const float nv = sample_n(rho, nx, ny, nz, sx + d.x * r, sy + d.y * r, sz + d.z * r, dx, inv_dx, pow2);
        const float inc = valid ? nv * nv * r * r * dr : 0.0f;
        float incl, excl, total, other = 0.0f;
        if (G == 1) {
            incl = inc;
            excl = 0.0f;
            total = inc;
        } else if (G == 2) {
            // one exchange gives the pair's scan: lane 1 adds lane 0's term (inc1 + inc0, the
            // general scan's operation) and both take that sum as the total
            other = __shfl_xor_sync(gmask, inc, 1, 2);
            incl = lane ? inc + other : inc;
            excl = lane ? other : 0.0f;
            total = lane ? incl : other + inc;
        } else {
            incl = inc;
#pragma unroll
            for (int o = 1; o < G; o <<= 1) {
                const float v = __shfl_up_sync(gmask, incl, o, G);
                if (lane >= o) incl = incl + v;
            }
            excl = __shfl_up_sync(gmask, incl, 1, G);
            if (lane == 0) excl = 0.0f;
            total = __shfl_sync(gmask, incl, G - 1, G);
        }
        const float col = hi + (excl - comp);
        const bool cross = valid && (col + inc > Q);
        const unsigned bal = __ballot_sync(0xffffffffu, cross);
        const unsigned mine = G == 32 ? bal : (bal >> ((threadIdx.x & 31) / G * G)) & ((1u << G) - 1u);
        float rfc = 0.0f;
        if (bal) {                               // some group of the warp crossed (warp-uniform)
            if (G <= 2) {
                // the pair's first crossing lane, from the terms both lanes hold
                const int p = G == 1 ? 0 : ((mine & 1u) ? 0 : 1);
                const float inc0 = lane ? other : inc;
                const float rp = ((float)(base + p) + 0.5f) * dr;
                const float colp = hi + ((p ? inc0 : 0.0f) - comp);
                const float incp = p == lane ? inc : other;
                rfc = rp - 0.5f * dr + dr * (Q - colp) / fmaxr(incp, 1e-20f);
            } else {
                const float rfl = r - 0.5f * dr + dr * (Q - col) / fmaxr(inc, 1e-20f);
                rfc = __shfl_sync(gmask, rfl, mine ? __ffs(mine) - 1 : 0, G);
            }
        }
        if (!done) {
            if (mine) {
                rf = rfc;
                done = true;
            } else {
                const float y = total - comp;
                const float tsum = hi + y;
                comp = (tsum - hi) - y;
                hi = tsum;
                done = base + G >= n1;
            }
        }
    }
    if (live && lane == 0) {
        float* p = reinterpret_cast<float*>(out & ~(uintptr_t)3);
        p[0] = rf;
        if (out & 1) p[-1] = rf;
        if (out & 2) p[1] = rf;
    }
}

// Where the front of ray (iu, ip) of star s goes in an instance's table [star][phi][u]: one float,
// or (pairs) the .x of its own float2 pair, flagged to write the .y of the pair below it too (and
// of its own at the last u).
__device__ __forceinline__ uintptr_t front_slot(float* rfront, bool pairs, int s, long long nray, int nu, int iu,
                                                int ip) {
    const long long e = (long long)s * nray + (long long)ip * nu + iu;
    if (!pairs) return reinterpret_cast<uintptr_t>(rfront + e);
    return reinterpret_cast<uintptr_t>(rfront + 2 * e) | (iu > 0 ? 1u : 0u) | (iu == nu - 1 ? 2u : 0u);
}

// Resident blocks per SM of the ray kernel: 5 (48 registers); at 6 (40 registers) the warp-uniform
// march spills 44-84 bytes.
#define NB_CAST_RAYS_MINB 5
template <int G, bool PAIRS>
__global__ void __launch_bounds__(256, NB_CAST_RAYS_MINB) cast_rays_kernel(const NbConst* __restrict__ c, const NbStarW* __restrict__ sw,
                                                        const float4* __restrict__ dirs,
                                                        const float* __restrict__ rho, float* __restrict__ rfront,
                                                        int nstars, const float* star_override, float q_override) {
    const int nray = c->nu * c->nphi;
    const long long gid = (blockIdx.x * (long long)blockDim.x + threadIdx.x) / G;
    const int lane = threadIdx.x % G;
    const unsigned gmask = G == 32 ? 0xffffffffu : (((1u << G) - 1u) << ((threadIdx.x & 31) / G * G));
    // no early exit: every lane of a warp reaches cast_ray's warp-uniform loop
    const bool in = gid < (long long)nray * nstars;
    // a group index of one instance stays below 2^32 (nb_create checks it): 32-bit division
    const unsigned g32 = in ? (unsigned)gid : 0u;
    const int s = (int)(g32 / (unsigned)nray), ray = (int)(g32 - (unsigned)s * (unsigned)nray);
    if (star_override) {
        cast_ray<G>(*c, dirs, rho, reinterpret_cast<uintptr_t>(rfront + ray), ray, star_override[0], star_override[1],
                    star_override[2], q_override, lane, gmask, in);
        return;
    }
    const NbStarW w = sw[s];
    // the instance's table is [star][phi][u] (u fastest: the cells of a warp share phi)
    const int iu = ray / c->nphi, ip = ray - iu * c->nphi;
    cast_ray<G>(*c, dirs, rho, front_slot(rfront, PAIRS, s, nray, c->nu, iu, ip), ray, w.w.x, w.w.y, w.w.z, w.q_f,
                lane, gmask, in && w.active);
}

// Rays of every star of every listed instance: job e owns groups [job[e].ray0, job[e+1].ray0).
// `J` holds the job records (global memory, or the kernel parameter of the param form); the active
// flags always come from `Jd`, the device copy (they change between replays of a captured step).
template <int G, typename Jobs>
__device__ __forceinline__ void cast_rays_batch_body(const Jobs& J, const NbRayJob* __restrict__ Jd, int n_jobs,
                                                     long long n_groups) {
    const long long gid0 = (blockIdx.x * (long long)blockDim.x + threadIdx.x) / G;
    const int lane = threadIdx.x % G;
    const unsigned gmask = G == 32 ? 0xffffffffu : (((1u << G) - 1u) << ((threadIdx.x & 31) / G * G));
    // no early exit: every lane of a warp reaches cast_ray's warp-uniform loop
    const bool in = gid0 < n_groups;
    const long long gid = in ? gid0 : 0;
    int lo = 0, hi = n_jobs - 1;
    while (lo < hi) {                          // last job with ray0 <= gid
        const int mid = (lo + hi + 1) >> 1;
        if (J[mid].ray0 <= gid) lo = mid; else hi = mid - 1;
    }
    const NbRayJob& job = J[lo];
    const NbConst& C = *job.c;
    const int nray = C.nu * C.nphi;
    const long long local = gid - job.ray0;
    const unsigned l32 = (unsigned)local;        // below 2^32 within a job (nb_create): 32-bit division
    const int s = (int)(l32 / (unsigned)nray), ray = (int)(l32 - (unsigned)s * (unsigned)nray);
    const bool star = in && s < job.nstars && Jd[lo].active;
    NbStarW w{};
    if (star) w = job.sw[s];
    const int iu = ray / C.nphi, ip = ray - iu * C.nphi;
    cast_ray<G>(C, job.dirs, job.rho, front_slot(job.rfront, job.pairs != 0, s, nray, C.nu, iu, ip), ray, w.w.x,
                w.w.y, w.w.z, w.q_f, lane, gmask, star && w.active);
}

template <int G>
__global__ void __launch_bounds__(256) cast_rays_batch_kernel(const NbRayJob* __restrict__ jobs, int n_jobs,
                                                              long long n_groups) {
    cast_rays_batch_body<G>(jobs, jobs, n_jobs, n_groups);
}

// the job records in the kernel parameter (constant bank): 48 registers, 5 blocks / SM
template <int G>
__global__ void __launch_bounds__(256, NB_CAST_RAYS_MINB)
    cast_rays_batch_param_kernel(const __grid_constant__ NbRayJobs P, const NbRayJob* __restrict__ jobs, int n_jobs,
                                 long long n_groups) {
    cast_rays_batch_body<G>(P.J, jobs, n_jobs, n_groups);
}

// The stars that can change xi or the front distance of the 32-cell segment [kb, kb + 32) of a
// row, as a mask (1 <= nstars <= NB_ROW_STARS).  Over the segment a star's
// r - rf lies in [LB, UB]: LB = (least distance to the segment) - (largest front radius of the
// star), UB = (largest distance) - (smallest front radius).  A star with LB at or above both
// min(1e3, least UB over the stars) and width / 2, plus a margin of one cell for float rounding,
// gives every cell of the segment val = 0 (no xi) and an r - rf above another star's (no front
// distance): leaving it out changes no bit.  A NaN bound (NaN radii or positions, whose min /
// max merges depend on order) keeps every active star.
// Computed for per_pass = 32 / nstars consecutive segments [kb0 + 32 g, kb0 + 32 g + 32) at once:
// lane g * nstars + s bounds star s over segment g, each segment's least upper bound is gathered
// from its nstars lanes, and lane g returns segment g's mask (bit s: star s).  One warp pass per
// per_pass segments: the culling costs ~per_pass times fewer instructions per cell.
__device__ __forceinline__ unsigned segment_masks(const float4* st, const int* act, const float4* tab,
                                                  const float2* bnd, int nstars, int kb0, int per_pass, int nz,
                                                  float dx, float width) {
    const int lane = threadIdx.x;
    const int g = lane / nstars, s = lane - g * nstars;
    const int kb = kb0 + 32 * g;
    const bool on = g < per_pass && kb < nz && act[s];
    float lb = __int_as_float(0x7f800000), ub = lb;       // +inf: the lane bounds no star
    bool bad = false;
    if (on) {
        const float sz = st[s].z, d2 = tab[s].x;
        const float2 b = bnd[s];                          // (least, largest) front radius
        const float z0 = ((float)kb + 0.5f) * dx, z1 = ((float)(min(kb + 31, nz - 1)) + 0.5f) * dx;
        const float en = fmaxf(0.0f, fmaxf(z0 - sz, sz - z1));
        const float ex = fmaxf(fabsf(sz - z0), fabsf(sz - z1));
        lb = sqrtf(d2 + en * en) - b.y;
        ub = sqrtf(d2 + ex * ex) - b.x;
        bad = isnan(lb) || isnan(ub);
    }
    const int base = min(g * nstars, 31);
    float m = __int_as_float(0x7f800000);
    for (int t = 0; t < nstars; ++t) m = fminf(m, __shfl_sync(0xffffffffu, ub, min(base + t, 31)));
    const float thr = fmaxf(fminf(1e3f, m), 0.5f * width) + dx;
    const unsigned keep = __ballot_sync(0xffffffffu, on && lb < thr);
    const unsigned all = __ballot_sync(0xffffffffu, on);
    const unsigned nan = __ballot_sync(0xffffffffu, bad);
    if (lane >= per_pass) return 0u;
    const int sh = lane * nstars;
    const unsigned full = nstars == 32 ? 0xffffffffu : ((1u << nstars) - 1u);
    return ((nan >> sh) & full) ? (all >> sh) & full : (keep >> sh) & full;
}

// nebula3d.py:273-307 rf_at + apply_front over one row (i, j), fused over the active stars,
// with the fp16 store of the front distance (sim.py:942, 980-985).  `tab`: this warp's row
// table (NB_ROW_STARS entries) or null for the per-cell form; `bnd`: each star's (least, largest)
// front radius, or null to merge every active star in every segment.  PAIRS: the front table
// holds (u, u + 1) pairs.
template <bool PAIRS>
__device__ __forceinline__ void apply_front_row(const NbConst& C, const float4* st, const int* act, int nstars,
                                                const float* __restrict__ rfront, float* __restrict__ xi_raw,
                                                void* __restrict__ dfront, bool half, int row, float4* tab,
                                                const float2* bnd) {
    const int nx = C.nx, ny = C.ny, nz = C.nz, nu = C.nu, nphi = C.nphi;
    if (row >= nx * ny) return;
    const int i = row / ny, j = row - (row / ny) * ny;
    const long long base = (long long)row * nz;
    const float dx = C.dx, width = C.width;
#if NB_ARITH_FAST
    const float inv_width = 1.0f / width;
#endif
    const float two_pi = 2.0f * pi_f();
    const float px = ((float)i + 0.5f) * dx, py = ((float)j + 0.5f) * dx;
    const long long rstride = (long long)nu * nphi;
    if (tab && nstars > NB_ROW_STARS) tab = nullptr;
    if (!tab) bnd = nullptr;
    if (tab) star_row_table(st, act, nstars, px, py, nphi, nu, tab);
    const unsigned row_stars = tab ? __ballot_sync(0xffffffffu, (int)threadIdx.x < nstars && act[threadIdx.x]) : 0u;
    constexpr int SG = 2;                       // stars whose gathers are in flight together
    // the culling masks of per_pass segments come from one pass (segment_masks): lane g holds
    // segment g's, broadcast when that segment's cells are merged
    if (nstars < 1) bnd = nullptr;
    const int per_pass = bnd ? 32 / nstars : 1;
    for (int kb0 = 0; kb0 < nz; kb0 += 32 * per_pass) {
      const unsigned masks = bnd ? segment_masks(st, act, tab, bnd, nstars, kb0, per_pass, nz, dx, width) : 0u;
      for (int g = 0; g < per_pass; ++g) {
        const int kb = kb0 + 32 * g;
        if (kb >= nz) break;                     // uniform over the warp
        const unsigned seg = bnd ? __shfl_sync(0xffffffffu, masks, g) : row_stars;
        const int k = kb + (int)threadIdx.x;
        if (k >= nz) continue;
        const long long q = base + k;
        const float pz = ((float)k + 0.5f) * dx;
        float xi = 0.0f, df = 1e3f;
        unsigned left = seg;                     // mask form: the segment's stars in star order
        for (int s0 = 0; tab ? left != 0u : s0 < nstars; s0 += SG) {
            float r[SG], tu[SG], tp[SG], g00[SG], g01[SG], g10[SG], g11[SG];
            bool on[SG];
#pragma unroll
            for (int e = 0; e < SG; ++e) {
                int s;
                if (tab) {
                    on[e] = left != 0u;
                    s = on[e] ? __ffs(left) - 1 : 0;
                    left &= left - 1u;
                } else {
                    s = s0 + e;
                    on[e] = s < nstars && act[s];
                }
                if (!on[e]) continue;                   // an empty slot's values are never read
                const float4 sp = st[s];
                const float* rfs = rfront + (long long)s * rstride;
                const float rz = pz - sp.z;
                int c0, c1;                      // phi columns times nu (table [phi][u])
                if (tab) {
                    const float4 tb = tab[s];
                    r[e] = fmaxq(sqrtf(tb.x + rz * rz), 1e-6f);                  // (rx^2 + ry^2) + rz^2
                    tp[e] = tb.y;
                    c0 = __float_as_int(tb.z);
                    c1 = __float_as_int(tb.w);
                } else {
                    const float rx = px - sp.x, ry = py - sp.y;
                    r[e] = fmaxq(sqrtf((rx * rx + ry * ry) + rz * rz), 1e-6f);     // 0 + x*x == x*x
                    float phi = atan2f(ry, rx);
                    if (phi < 0.0f) phi = phi + two_pi;
                    const float fp = phi / two_pi * (float)nphi - 0.5f;
                    const int ip = (int)floorf(fp);
                    tp[e] = fp - (float)ip;
                    c0 = wrap_index(ip, nphi) * nu;
                    c1 = wrap_index(ip + 1, nphi) * nu;
                }
#if NB_ARITH_FAST
                const float u = rz * rcp_approx(r[e]);
#else
                const float u = rz / r[e];
#endif
                const float fu = (u + 1.0f) * 0.5f * (float)nu - 0.5f;
                const int iu = (int)floorf(fu);
                tu[e] = fu - (float)iu;
                const int u0 = max(iu, 0), u1 = min(iu + 1, nu - 1);    // u in [-1, 1]: iu in [-1, nu - 1]
                if (PAIRS) {
                    // pair u0 = (rf(u0), rf(min(u0 + 1, nu - 1))): the two u corners, except at iu = -1,
                    // where both corners clamp to u = 0 (the pair's .x)
                    const float2* rp = reinterpret_cast<const float2*>(rfront) + (long long)s * rstride;
                    const float2 p0 = __ldg(rp + c0 + u0), p1 = __ldg(rp + c1 + u0);
                    g00[e] = p0.x;
                    g01[e] = p1.x;
                    g10[e] = iu < 0 ? p0.x : p0.y;
                    g11[e] = iu < 0 ? p1.x : p1.y;
                } else {
                    g00[e] = __ldg(rfs + c0 + u0);
                    g01[e] = __ldg(rfs + c1 + u0);
                    g10[e] = __ldg(rfs + c0 + u1);
                    g11[e] = __ldg(rfs + c1 + u1);
                }
            }
#pragma unroll
            for (int e = 0; e < SG; ++e) {
                if (!on[e]) continue;
                const float ra = g00[e] * (1.0f - tp[e]) + g01[e] * tp[e];
                const float rb = g10[e] * (1.0f - tp[e]) + g11[e] * tp[e];
                const float rf = ra * (1.0f - tu[e]) + rb * tu[e];
#if NB_ARITH_FAST
                // clamped to [0, 1] by the saturating form of the multiply-add; merged by one max
                xi = fmaxf(xi, __saturatef((rf - r[e]) * inv_width + 0.5f));
#else
                const float val = fminr(fmaxr(0.0f, (rf - r[e]) / width + 0.5f), 1.0f);
                if (val > xi) xi = val;              // in star order, as the reference merges
#endif
                df = fminq(df, r[e] - rf);
            }
        }
        if (C.plane_on) {                        // the -x plane-parallel source: same merge rules
            const float xf = __ldg(C.plane_xf + (long long)j * nz + k);
            const float val = fminr(fmaxr(0.0f, (xf - px) / width + 0.5f), 1.0f);
            if (val > xi) xi = val;
            df = fminr(df, px - xf);
        }
        xi_raw[q] = xi;
        if (half)
            reinterpret_cast<__half*>(dfront)[q] = __float2half_rn(df);
        else
            reinterpret_cast<float*>(dfront)[q] = df;
      }
    }
}

// Each active star's least and largest front radius over its rays, as NB_FRONT_PARTS partial
// (least, largest) pairs per star: block (b, s) reduces the b-th slice of star s.  The largest is
// NaN when a NaN radius was seen (the least skips NaNs).
// With pair tables a star's slice holds every front twice (as a .x and as a .y): the same set of
// values, so the same bounds.
__device__ __forceinline__ void front_bounds_block(const NbStarW* __restrict__ sw, const float* __restrict__ rfront,
                                                   long long nray, float2* __restrict__ parts, int s, int b) {
    if (!sw[s].active) return;                  // uniform over the block
    const float* r = rfront + (long long)s * nray;
    const long long per = (nray + NB_FRONT_PARTS - 1) / NB_FRONT_PARTS;
    const long long lo = (long long)b * per, hi = min(nray, lo + per);
    float mn = __int_as_float(0x7f800000), mx = -mn;
    bool nan = false;
    for (long long q = lo + threadIdx.x; q < hi; q += blockDim.x) {
        const float v = __ldg(r + q);
        nan |= isnan(v);
        mn = fminf(mn, v);
        mx = fmaxf(mx, v);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        mn = fminf(mn, __shfl_xor_sync(0xffffffffu, mn, o));
        mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    }
    __shared__ float2 wpart[8];
    const bool any_nan = __syncthreads_or(nan);
    if ((threadIdx.x & 31) == 0) wpart[threadIdx.x >> 5] = make_float2(mn, mx);
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < (int)(blockDim.x >> 5); ++w) {
            mn = fminf(mn, wpart[w].x);
            mx = fmaxf(mx, wpart[w].y);
        }
        parts[s * NB_FRONT_PARTS + b] = make_float2(mn, any_nan ? __int_as_float(0x7fc00000) : mx);
    }
}

__global__ void __launch_bounds__(256) front_bounds_kernel(const NbStarW* __restrict__ sw,
                                                           const float* __restrict__ rfront, long long nray,
                                                           float2* __restrict__ parts) {
    front_bounds_block(sw, rfront, nray, parts, blockIdx.y, blockIdx.x);
}

// the same for every listed instance that culls: block (b, job, star)
__global__ void __launch_bounds__(256) front_bounds_batch_kernel(const NbRayJob* __restrict__ jobs) {
    const NbRayJob& J = jobs[blockIdx.y];
    if (!J.front_parts || !J.active || (int)blockIdx.z >= J.nstars) return;      // uniform over the block
    front_bounds_block(J.sw, J.rfront, J.pairs ? 2 * J.nray : J.nray, J.front_parts, blockIdx.z, blockIdx.x);
}

// the partials into (least, largest) per star in shared memory (after load_stars' barrier)
__device__ __forceinline__ void load_front_bounds(const float2* parts, int nstars, float2* bnd, int tlin) {
    for (int s = tlin; s < nstars; s += blockDim.x * blockDim.y) {
        float mn = __int_as_float(0x7f800000), mx = -mn;
        bool nan = false;
        for (int b = 0; b < NB_FRONT_PARTS; ++b) {
            const float2 p = parts[s * NB_FRONT_PARTS + b];
            mn = fminf(mn, p.x);
            nan |= isnan(p.y);
            mx = fmaxf(mx, p.y);
        }
        bnd[s] = make_float2(mn, nan ? __int_as_float(0x7fc00000) : mx);
    }
    __syncthreads();
}

__device__ __forceinline__ int load_stars(const NbStarW* sw, int nstars, float4* st, int* act) {
    const int tlin = threadIdx.y * blockDim.x + threadIdx.x;
    for (int s = tlin; s < nstars; s += blockDim.x * blockDim.y) {
        st[s] = sw[s].w;
        act[s] = sw[s].active;
    }
    __syncthreads();
    return tlin;
}

template <bool HALF, bool PAIRS>
__global__ void __launch_bounds__(256, 4) apply_front_kernel(const NbConst* __restrict__ c,
                                                          const NbStarW* __restrict__ sw,
                                                          const float* __restrict__ rfront, int nstars,
                                                          float* __restrict__ xi_raw, void* __restrict__ dfront,
                                                          unsigned* smax_reset, const float2* __restrict__ parts) {
    __shared__ float4 st[NB_MAX_STARS];
    __shared__ int act[NB_MAX_STARS];
    __shared__ float4 tab[8][NB_ROW_STARS];
    __shared__ float2 bnd[NB_ROW_STARS];
    const int tlin = load_stars(sw, nstars, st, act);
    if (smax_reset && blockIdx.x == 0 && tlin == 0) *smax_reset = 0u;
    if (parts) load_front_bounds(parts, nstars, bnd, tlin);      // parts only with nstars <= NB_ROW_STARS
    apply_front_row<PAIRS>(*c, st, act, nstars, rfront, xi_raw, dfront, HALF, blockIdx.x * blockDim.y + threadIdx.y,
                           tab[threadIdx.y], parts ? bnd : nullptr);
}

// Rows of every listed instance; job e owns blocks [job[e].blk0, job[e+1].blk0) (8 rows each).
__global__ void __launch_bounds__(256) apply_front_batch_kernel(const NbRayJob* __restrict__ jobs, int n_jobs) {
    __shared__ float4 st[NB_MAX_STARS];
    __shared__ int act[NB_MAX_STARS];
    __shared__ float4 tab[8][NB_ROW_STARS];
    __shared__ float2 bnd[NB_ROW_STARS];
    int lo = 0, hi = n_jobs - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (jobs[mid].blk0 <= (long long)blockIdx.x) lo = mid; else hi = mid - 1;
    }
    const NbRayJob& J = jobs[lo];
    if (!J.active) return;                       // uniform over the block
    const int lb = (int)(blockIdx.x - J.blk0);
    const int tlin = load_stars(J.sw, J.nstars, st, act);
    if (lb == 0 && tlin == 0) *J.smax = 0u;
    if (J.front_parts) load_front_bounds(J.front_parts, J.nstars, bnd, tlin);     // uniform over the block
    if (J.pairs)
        apply_front_row<true>(*J.c, st, act, J.nstars, J.rfront, J.xi_raw, J.dfront, J.half != 0,
                              lb * blockDim.y + threadIdx.y, tab[threadIdx.y], J.front_parts ? bnd : nullptr);
    else
        apply_front_row<false>(*J.c, st, act, J.nstars, J.rfront, J.xi_raw, J.dfront, J.half != 0,
                               lb * blockDim.y + threadIdx.y, tab[threadIdx.y], J.front_parts ? bnd : nullptr);
}

// nebula3d.py:310-315 smooth_xi (+ sim.py:941 copy back) of one row, then the CFL max speed
// (nebula3d.py:154-162) of the state with the new xi.
__device__ __forceinline__ float smooth_row(const NbConst& C, const float* __restrict__ src, float* __restrict__ xi,
                                            const float* __restrict__ rho, const float* __restrict__ mx,
                                            const float* __restrict__ my, const float* __restrict__ mz, bool smax,
                                            int row) {
    const int nx = C.nx, ny = C.ny, nz = C.nz;
    const float cn2 = C.cn2, ci2 = C.ci2;
    float m = 0.0f;
    if (row >= nx * ny) return m;
    const int i = row / ny, j = row - (row / ny) * ny;
    const long long base = (long long)row * nz;
    const long long sj = nz, si = (long long)ny * nz;
    const long long dxm = i > 0 ? si : 0, dxp = i < nx - 1 ? si : 0;
    const long long dym = j > 0 ? sj : 0, dyp = j < ny - 1 ? sj : 0;
#pragma unroll 4
    for (int k = threadIdx.x; k < nz; k += 32) {
        const long long q = base + k;
        const float xm = __ldg(src + q - dxm), xp = __ldg(src + q + dxp);
        const float ym = __ldg(src + q - dym), yp = __ldg(src + q + dyp);
        const float zm = __ldg(src + q - (k > 0 ? 1 : 0)), zp = __ldg(src + q + (k < nz - 1 ? 1 : 0));
        const float mm = (xm + xp + ym + yp + zm + zp) / 6.0f;
        const float x = 0.5f * __ldg(src + q) + 0.5f * mm;
        xi[q] = x;
        if (smax) {
            const float r = rho[q];
#if NB_ARITH_FAST
            const float ri = 1.0f / r;               // one division for the three velocities
            const float v = fabsf(mx[q] * ri) + fabsf(my[q] * ri) + fabsf(mz[q] * ri) + sqrtf(cn2 + x * (ci2 - cn2));
#else
            const float v = fabsf(mx[q] / r) + fabsf(my[q] / r) + fabsf(mz[q] / r) + sqrtf(cn2 + x * (ci2 - cn2));
#endif
            m = fmaxr(v, m);
        }
    }
    return m;
}

__device__ __forceinline__ void block_max_to(float m, unsigned* smax_bits) {
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

__global__ void __launch_bounds__(256) smooth_kernel(const NbConst* __restrict__ c, const float* __restrict__ src,
                                                     float* __restrict__ xi, const float* __restrict__ rho,
                                                     const float* __restrict__ mx, const float* __restrict__ my,
                                                     const float* __restrict__ mz, unsigned* smax_bits) {
    const float m = smooth_row(*c, src, xi, rho, mx, my, mz, smax_bits != nullptr,
                               blockIdx.x * blockDim.y + threadIdx.y);
    if (smax_bits) block_max_to(m, smax_bits);
}

__global__ void __launch_bounds__(256) smooth_batch_kernel(const NbRayJob* __restrict__ jobs, int n_jobs) {
    int lo = 0, hi = n_jobs - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (jobs[mid].blk0 <= (long long)blockIdx.x) lo = mid; else hi = mid - 1;
    }
    const NbRayJob& J = jobs[lo];
    if (!J.active) return;                       // uniform over the block
    const int lb = (int)(blockIdx.x - J.blk0);
    const float m = smooth_row(*J.c, J.xi_raw, J.xi, J.rho, J.mx, J.my, J.mz, true, lb * blockDim.y + threadIdx.y);
    block_max_to(m, J.smax);
}

// Plane-parallel ionizing source on the -x face (no reference counterpart): per (j,k) column, the
// recombination column sum n^2 dx along +x in cell order, the front where it passes the flux F,
// interpolated inside the crossing cell as cast_rays does (nebula3d.py:262-268); no front: rcap.
__global__ void __launch_bounds__(256) plane_front_kernel(const NbConst* __restrict__ c, const float* __restrict__ rho,
                                                          float* __restrict__ xf) {
    const int nx = c->nx, ny = c->ny, nz = c->nz;
    const int col = blockIdx.x * blockDim.x + threadIdx.x;
    if (col >= ny * nz) return;
    const float F = c->plane_F_f, dx = c->dx;
    float sum = 0.0f, x = c->diag_f;
    const long long plane = (long long)ny * nz;
    for (int i = 0; i < nx; ++i) {
        const float n = __ldg(rho + i * plane + col);
        const float inc = n * n * dx;
        if (sum + inc > F) {
            x = ((float)i + 0.5f) * dx - 0.5f * dx + dx * (F - sum) / fmaxr(inc, 1e-20f);
            break;
        }
        sum = sum + inc;
    }
    xf[col] = x;
}

}  // namespace

cudaError_t nb_launch_plane_front(const NbConst* c, const float* rho, float* xf, int ny, int nz, cudaStream_t s) {
    const int cols = ny * nz;
    plane_front_kernel<<<(cols + 255) / 256, 256, 0, s>>>(c, rho, xf);
    return cudaGetLastError();
}

cudaError_t nb_launch_ray_dirs(int nu, int nphi, float4* dirs, cudaStream_t s) {
    const int n = nu * nphi;
    ray_dirs_kernel<<<(n + 255) / 256, 256, 0, s>>>(nu, nphi, dirs);
    return cudaGetLastError();
}

cudaError_t nb_launch_cast_rays(const NbConst* c, const NbStarW* sw, const float4* dirs, const float* rho,
                                float* rfront, int nstars, int group, const float* star_override, float q_override,
                                cudaStream_t s, int nu, int nphi, int pairs) {
    const long long threads = (long long)nu * nphi * nstars * group;
    const int blocks = (int)((threads + 255) / 256);
#define NB_RAYS_LAUNCH(G)                                                                                      \
    (pairs ? cast_rays_kernel<G, true><<<blocks, 256, 0, s>>>(c, sw, dirs, rho, rfront, nstars, star_override,  \
                                                              q_override)                                       \
           : cast_rays_kernel<G, false><<<blocks, 256, 0, s>>>(c, sw, dirs, rho, rfront, nstars, star_override, \
                                                               q_override))
    switch (group) {
        case 1: NB_RAYS_LAUNCH(1); break;
        case 2: NB_RAYS_LAUNCH(2); break;
        case 4: NB_RAYS_LAUNCH(4); break;
        case 8: NB_RAYS_LAUNCH(8); break;
        case 16: NB_RAYS_LAUNCH(16); break;
        default: NB_RAYS_LAUNCH(32); break;
    }
#undef NB_RAYS_LAUNCH
    return cudaGetLastError();
}

cudaError_t nb_launch_apply_front(const NbConst* c, const NbStarW* sw, const float* rfront, int nstars,
                                  float* xi_raw, void* dfront, unsigned* smax_reset, cudaStream_t s, int nx, int ny,
                                  int half, float2* front_parts, long long nray, int pairs) {
    const dim3 blk(32, 8);
    const int blocks = rowwalk_blocks(nx, ny);
    const float2* parts = nullptr;
    if (front_parts && nstars >= 1 && nstars <= NB_ROW_STARS) {
        front_bounds_kernel<<<dim3(NB_FRONT_PARTS, nstars), 256, 0, s>>>(sw, rfront, pairs ? 2 * nray : nray,
                                                                          front_parts);
        parts = front_parts;
    }
    if (half && pairs)
        apply_front_kernel<true, true><<<blocks, blk, 0, s>>>(c, sw, rfront, nstars, xi_raw, dfront, smax_reset, parts);
    else if (half)
        apply_front_kernel<true, false><<<blocks, blk, 0, s>>>(c, sw, rfront, nstars, xi_raw, dfront, smax_reset, parts);
    else if (pairs)
        apply_front_kernel<false, true><<<blocks, blk, 0, s>>>(c, sw, rfront, nstars, xi_raw, dfront, smax_reset, parts);
    else
        apply_front_kernel<false, false><<<blocks, blk, 0, s>>>(c, sw, rfront, nstars, xi_raw, dfront, smax_reset, parts);
    return cudaGetLastError();
}

cudaError_t nb_launch_smooth(const NbConst* c, const float* xi_raw, float* xi, const float* rho, const float* mx,
                             const float* my, const float* mz, unsigned* smax_bits, cudaStream_t s, int nx, int ny) {
    smooth_kernel<<<rowwalk_blocks(nx, ny), dim3(32, 8), 0, s>>>(c, xi_raw, xi, rho, mx, my, mz, smax_bits);
    return cudaGetLastError();
}

cudaError_t nb_launch_ionize_batch(const NbRayJob* jobs, const NbRayJob* host_jobs, int n_jobs, long long n_groups,
                                   long long n_blocks, int group, cudaStream_t s) {
    if (n_jobs <= 0) return cudaSuccess;
    const long long threads = n_groups * group;
    const long long blocks = (threads + 255) / 256;
    if (blocks > 0 && host_jobs && n_jobs <= NB_BATCH_PARAM_MAX) {
        NbRayJobs P;
        std::memset(&P, 0, sizeof(P));
        std::memcpy(P.J, host_jobs, sizeof(NbRayJob) * n_jobs);
        const unsigned nb = (unsigned)blocks;
        switch (group) {
            case 1: cast_rays_batch_param_kernel<1><<<nb, 256, 0, s>>>(P, jobs, n_jobs, n_groups); break;
            case 2: cast_rays_batch_param_kernel<2><<<nb, 256, 0, s>>>(P, jobs, n_jobs, n_groups); break;
            case 4: cast_rays_batch_param_kernel<4><<<nb, 256, 0, s>>>(P, jobs, n_jobs, n_groups); break;
            case 8: cast_rays_batch_param_kernel<8><<<nb, 256, 0, s>>>(P, jobs, n_jobs, n_groups); break;
            case 16: cast_rays_batch_param_kernel<16><<<nb, 256, 0, s>>>(P, jobs, n_jobs, n_groups); break;
            default: cast_rays_batch_param_kernel<32><<<nb, 256, 0, s>>>(P, jobs, n_jobs, n_groups); break;
        }
    } else if (blocks > 0) {
        switch (group) {
            case 1: cast_rays_batch_kernel<1><<<(unsigned)blocks, 256, 0, s>>>(jobs, n_jobs, n_groups); break;
            case 2: cast_rays_batch_kernel<2><<<(unsigned)blocks, 256, 0, s>>>(jobs, n_jobs, n_groups); break;
            case 4: cast_rays_batch_kernel<4><<<(unsigned)blocks, 256, 0, s>>>(jobs, n_jobs, n_groups); break;
            case 8: cast_rays_batch_kernel<8><<<(unsigned)blocks, 256, 0, s>>>(jobs, n_jobs, n_groups); break;
            case 16: cast_rays_batch_kernel<16><<<(unsigned)blocks, 256, 0, s>>>(jobs, n_jobs, n_groups); break;
            default: cast_rays_batch_kernel<32><<<(unsigned)blocks, 256, 0, s>>>(jobs, n_jobs, n_groups); break;
        }
    }
    front_bounds_batch_kernel<<<dim3(NB_FRONT_PARTS, n_jobs, NB_ROW_STARS), 256, 0, s>>>(jobs);
    apply_front_batch_kernel<<<(unsigned)n_blocks, dim3(32, 8), 0, s>>>(jobs, n_jobs);
    smooth_batch_kernel<<<(unsigned)n_blocks, dim3(32, 8), 0, s>>>(jobs, n_jobs);
    return cudaGetLastError();
}
