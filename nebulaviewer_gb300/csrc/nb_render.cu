// The renderer's voxel pack: the consumer of rho / xi / dfront / g0 on the display side.
//
//  * render.py:176-205 pack_volume_lm: per cell an RGBA16F voxel (emission r, g, b; dust) from
//    the line mix of the Blender "Nebula Volume" shader (render.py:3-8): ha = (rho xi)^2,
//    OIII and SII = ha weighted by smoothsteps of dfront, dust = rho (1 - xi) + 0.08 rho xi,
//    the FUV term dust * (g0 / (1 + g0 / Gs) + ambient), the shock proxy (nebula3d.py:182-191)
//    computed inline, each times its palette colour; a soft fade near the box faces; min(., 6e4)
//    and round-to-nearest-even float16.
//  * render.py:281-298 smooth_axis: the [1 4 1]/6 prefilter along x, then y, then z.
// The voxel grid is C-order (nx, ny, nz, 4) float16: one 8-byte store per cell, so a warp writes
// 256 contiguous bytes.  The texture upload and the ray marcher that read it are display work
// (no graphics stack on this machine); the pack leaves a device buffer.
#include "nb_rayutil.cuh"

namespace {

// render.py:127-131 sstep
__device__ __forceinline__ float sstep(float e0, float e1, float x) {
    const float t = fminr(fmaxr(0.0f, (x - e0) / (e1 - e0)), 1.0f);
    return t * t * (3.0f - 2.0f * t);
}

// render.py:135-139 fade_axis
__device__ __forceinline__ float fade_axis(float u, float e) {
    if (e <= 0.0f) return 1.0f;
    return sstep(0.0f, e, u) * sstep(0.0f, e, 1.0f - u);
}

__device__ __forceinline__ unsigned half_bits(float v) { return (unsigned)__half_as_ushort(__float2half_rn(v)); }
__device__ __forceinline__ float half_lo(unsigned w) { return __half2float(__ushort_as_half((unsigned short)(w & 0xffffu))); }
__device__ __forceinline__ float half_hi(unsigned w) { return __half2float(__ushort_as_half((unsigned short)(w >> 16))); }

__device__ __forceinline__ float ld_any(const void* p, long long q, bool half) {
    return half ? __half2float(reinterpret_cast<const __half*>(p)[q]) : reinterpret_cast<const float*>(p)[q];
}

__global__ void __launch_bounds__(256) pack_kernel(const NbConst* __restrict__ c, const float* __restrict__ rho,
                                                   const float* __restrict__ mx, const float* __restrict__ my,
                                                   const float* __restrict__ mz, const float* __restrict__ xi,
                                                   const void* __restrict__ dfront, const void* __restrict__ g0,
                                                   bool half, const nb_pack_params pp, int shock_on,
                                                   uint2* __restrict__ out) {
    const NbConst& C = *c;
    const RowWalk w(C.nx, C.ny, C.nz);
    if (!w.valid) return;
    const float e = pp.edge, dx = pp.dx, m = 60000.0f;
    const float p0 = ((float)w.i + 0.5f) * dx * pp.inv_L[0];
    const float p1 = ((float)w.j + 0.5f) * dx * pp.inv_L[1];
    const float f01 = fade_axis(p0, e) * fade_axis(p1, e);
    for (int k = w.k0; k < C.nz; k += 32) {
        const long long q = w.base + k;
        const float r = rho[q];
        const float x = fminr(fmaxr(0.0f, xi[q]), 1.0f);
        const float df = ld_any(dfront, q, half);
        const float ni = r * x;
        const float ha = ni * ni;
        const float oiii = ha * sstep(-0.03f, -0.12f, df);
        const float sii = ha * sstep(-0.05f, -0.005f, df);
        float dust = r * (1.0f - x) + 0.08f * ni;
        const float g = ld_any(g0, q, half);
        const float geff = g / (1.0f + g / pp.gs) + pp.ambient;
        const float sh = shock_on ? nb_shock_at(C, rho, mx, my, mz, w.i, w.j, k) : 0.0f;
        const float dg = dust * geff;
        float em[3];
#pragma unroll
        for (int ch = 0; ch < 3; ++ch)
            em[ch] = ha * pp.c_ha[ch] + oiii * pp.c_o3[ch] + sii * pp.c_s2[ch] + dg * pp.c_dg[ch] + sh * pp.c_sh[ch];
        const float p2 = ((float)k + 0.5f) * dx * pp.inv_L[2];
        const float f = f01 * fade_axis(p2, e);
#pragma unroll
        for (int ch = 0; ch < 3; ++ch) em[ch] = em[ch] * f;
        dust = dust * f;
        out[q] = make_uint2(half_bits(fminr(em[0], m)) | (half_bits(fminr(em[1], m)) << 16),
                            half_bits(fminr(em[2], m)) | (half_bits(fminr(dust, m)) << 16));
    }
}

__global__ void __launch_bounds__(256) smooth_kernel(const NbConst* __restrict__ c, const uint2* __restrict__ src,
                                                     uint2* __restrict__ dst, int axis) {
    const NbConst& C = *c;
    const RowWalk w(C.nx, C.ny, C.nz);
    if (!w.valid) return;
    const long long si = (long long)C.ny * C.nz, sj = C.nz;
    const long long dm = axis == 0 ? (w.i > 0 ? si : 0) : (axis == 1 ? (w.j > 0 ? sj : 0) : 0);
    const long long dp = axis == 0 ? (w.i < C.nx - 1 ? si : 0) : (axis == 1 ? (w.j < C.ny - 1 ? sj : 0) : 0);
    for (int k = w.k0; k < C.nz; k += 32) {
        const long long q = w.base + k;
        const long long qa = axis == 2 ? (k > 0 ? q - 1 : q) : q - dm;
        const long long qc = axis == 2 ? (k < C.nz - 1 ? q + 1 : q) : q + dp;
        const uint2 a = __ldg(src + qa), b = __ldg(src + q), cc = __ldg(src + qc);
        const unsigned av[2] = {a.x, a.y}, bv[2] = {b.x, b.y}, cv[2] = {cc.x, cc.y};
        unsigned o[2];
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const float lo = (half_lo(av[h]) + 4.0f * half_lo(bv[h]) + half_lo(cv[h])) / 6.0f;
            const float hi = (half_hi(av[h]) + 4.0f * half_hi(bv[h]) + half_hi(cv[h])) / 6.0f;
            o[h] = half_bits(lo) | (half_bits(hi) << 16);
        }
        dst[q] = make_uint2(o[0], o[1]);
    }
}

}  // namespace

cudaError_t nb_launch_render_pack(const NbConst* c, const float* rho, const float* mx, const float* my, const float* mz,
                                  const float* xi, const void* dfront, const void* g0, int half,
                                  const nb_pack_params& pp, int shock_on, int smooth, void* out8, void* tmp8, int nx,
                                  int ny, cudaStream_t s) {
    const dim3 grid(rowwalk_blocks(nx, ny)), block(32, 8);
    uint2* out = static_cast<uint2*>(out8);
    uint2* tmp = static_cast<uint2*>(tmp8);
    // render.py:725-728: packed -> x -> packed2 -> y -> packed -> z -> packed2; here the result lands in `out`
    pack_kernel<<<grid, block, 0, s>>>(c, rho, mx, my, mz, xi, dfront, g0, half != 0, pp, shock_on, smooth ? tmp : out);
    if (smooth) {
        smooth_kernel<<<grid, block, 0, s>>>(c, tmp, out, 0);
        smooth_kernel<<<grid, block, 0, s>>>(c, out, tmp, 1);
        smooth_kernel<<<grid, block, 0, s>>>(c, tmp, out, 2);
    }
    return cudaGetLastError();
}
