// Device helpers shared by the ray kernels (ionizing rays and FUV rays).
#pragma once
#include "nb_internal.cuh"

__device__ __forceinline__ float pi_f() { return 3.14159265358979323846f; }

// nebula3d.py:195-226 sample_n (trilinear, 0 outside the domain), without branches: the corners
// are always clamped to the grid (no-ops inside it) and 0 is selected outside the domain, so the
// lanes of a warp never diverge here.  With dx == 2^-m the division p / dx is the exact
// multiplication p * 2^m.  A plane ny * nz stays below 2^31 cells (nb_create requires it).
__device__ __forceinline__ float sample_n(const float* __restrict__ a, int nx, int ny, int nz, float px, float py,
                                          float pz, float dx, float inv_dx, bool pow2) {
    const float gx = (pow2 ? px * inv_dx : px / dx) - 0.5f;
    const float gy = (pow2 ? py * inv_dx : py / dx) - 0.5f;
    const float gz = (pow2 ? pz * inv_dx : pz / dx) - 0.5f;
    const bool outside = gx < -0.5f || gy < -0.5f || gz < -0.5f || gx > (float)nx - 0.5f || gy > (float)ny - 0.5f ||
                         gz > (float)nz - 0.5f;
    const float fgx = floorf(gx), fgy = floorf(gy), fgz = floorf(gz);
    const int i0 = (int)fgx, j0 = (int)fgy, k0 = (int)fgz;
    const float fx = gx - (float)i0, fy = gy - (float)j0, fz = gz - (float)k0;
    const int ia = iclampd(i0, 0, nx - 1), ib = iclampd(i0 + 1, 0, nx - 1);
    const int ja = iclampd(j0, 0, ny - 1), jb = iclampd(j0 + 1, 0, ny - 1);
    const int ka = iclampd(k0, 0, nz - 1), kb = iclampd(k0 + 1, 0, nz - 1);
    const float* p = a + (((long long)ia * ny + ja) * nz + ka);
    const int dk = kb - ka, dj = (jb - ja) * nz, di = (ib - ia) * (ny * nz);
    const float c000 = __ldg(p), c100 = __ldg(p + di);
    const float c010 = __ldg(p + dj), c110 = __ldg(p + (di + dj));
    const float c001 = __ldg(p + dk), c101 = __ldg(p + (di + dk));
    const float c011 = __ldg(p + (dj + dk)), c111 = __ldg(p + (di + dj + dk));
    const float c00 = c000 + (c100 - c000) * fx;
    const float c10 = c010 + (c110 - c010) * fx;
    const float c01 = c001 + (c101 - c001) * fx;
    const float c11 = c011 + (c111 - c011) * fx;
    const float c0 = c00 + (c10 - c00) * fy;
    const float c1 = c01 + (c11 - c01) * fy;
    const float v = c0 + (c1 - c0) * fz;
    return outside ? 0.0f : v;
}

// an approximate reciprocal (<= 1 ulp), for the fast build's divisions by a clamped distance
__device__ __forceinline__ float rcp_approx(float x) {
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

// sample_n of two fields stored interleaved ((rho, xi) pairs): the same corners, weights and
// float operations per field as two sample_n calls, with one 8-byte load per corner.
__device__ __forceinline__ float2 sample_n2(const float2* __restrict__ a, int nx, int ny, int nz, float px, float py,
                                           float pz, float dx, float inv_dx, bool pow2) {
    const float gx = (pow2 ? px * inv_dx : px / dx) - 0.5f;
    const float gy = (pow2 ? py * inv_dx : py / dx) - 0.5f;
    const float gz = (pow2 ? pz * inv_dx : pz / dx) - 0.5f;
    if (gx < -0.5f || gy < -0.5f || gz < -0.5f) return make_float2(0.0f, 0.0f);
    if (gx > (float)nx - 0.5f || gy > (float)ny - 0.5f || gz > (float)nz - 0.5f) return make_float2(0.0f, 0.0f);
    const int i0 = (int)floorf(gx), j0 = (int)floorf(gy), k0 = (int)floorf(gz);
    const float fx = gx - (float)i0, fy = gy - (float)j0, fz = gz - (float)k0;
    const int ia = iclampd(i0, 0, nx - 1), ib = iclampd(i0 + 1, 0, nx - 1);
    const int ja = iclampd(j0, 0, ny - 1), jb = iclampd(j0 + 1, 0, ny - 1);
    const int ka = iclampd(k0, 0, nz - 1), kb = iclampd(k0 + 1, 0, nz - 1);
    // as sample_n, always in the clamped form (an all-inside fast path measured slower in the FUV rays)
    const float2* p = a + (((long long)ia * ny + ja) * nz + ka);
    const int dk = kb - ka, dj = (jb - ja) * nz, di = (ib - ia) * (ny * nz);
    const float2 c000 = __ldg(p), c100 = __ldg(p + di);
    const float2 c010 = __ldg(p + dj), c110 = __ldg(p + (di + dj));
    const float2 c001 = __ldg(p + dk), c101 = __ldg(p + (di + dk));
    const float2 c011 = __ldg(p + (dj + dk)), c111 = __ldg(p + (di + dj + dk));
    float out[2];
#pragma unroll
    for (int f = 0; f < 2; ++f) {
        const float v000 = f ? c000.y : c000.x, v100 = f ? c100.y : c100.x, v010 = f ? c010.y : c010.x;
        const float v110 = f ? c110.y : c110.x, v001 = f ? c001.y : c001.x, v101 = f ? c101.y : c101.x;
        const float v011 = f ? c011.y : c011.x, v111 = f ? c111.y : c111.x;
        const float c00 = v000 + (v100 - v000) * fx;
        const float c10 = v010 + (v110 - v010) * fx;
        const float c01 = v001 + (v101 - v001) * fx;
        const float c11 = v011 + (v111 - v011) * fx;
        const float c0 = c00 + (c10 - c00) * fy;
        const float c1 = c01 + (c11 - c01) * fy;
        out[f] = c0 + (c1 - c0) * fz;
    }
    return make_float2(out[0], out[1]);
}

// nebula3d.py:229-244 box_range
__device__ __forceinline__ void nb_box_range(float ox, float oy, float oz, float dxr, float dyr, float dzr, const float* bmax,
                             float& t0, float& t1) {
    t0 = 0.0f;
    t1 = 1e9f;
    const float o[3] = {ox, oy, oz}, d[3] = {dxr, dyr, dzr};
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        if (fabsf(d[a]) < 1e-9f) {
            if (o[a] < 0.0f || o[a] > bmax[a]) t1 = -1.0f;
        } else {
            const float ta = (0.0f - o[a]) / d[a];
            const float tb = (bmax[a] - o[a]) / d[a];
            t0 = fmaxr(t0, fminr(ta, tb));
            t1 = fminr(t1, fmaxr(ta, tb));
        }
    }
}

// Python int() of a float32 (truncation), kept inside the int range
__device__ __forceinline__ int trunc_i(float x) {
    return x > 2e9f ? 2000000000 : (x < -2e9f ? -2000000000 : (int)x);
}

// Row-major cell walk for the per-cell kernels: blockDim = (32, 8); a thread owns row
// r = blockIdx.x * 8 + threadIdx.y (r = i * ny + j) and cells k = threadIdx.x + 32 m.
// One 32-bit division per thread instead of 64-bit divisions per cell.
struct RowWalk {
    int i, j, k0;
    long long base;       // linear index of (i, j, 0)
    bool valid;
    __device__ __forceinline__ RowWalk(int nx, int ny, int nz) {
        const int r = blockIdx.x * blockDim.y + threadIdx.y;
        valid = r < nx * ny;
        i = valid ? r / ny : 0;
        j = valid ? r - i * ny : 0;
        k0 = threadIdx.x;
        base = (long long)r * nz;
    }
};
__host__ __forceinline__ int rowwalk_blocks(int nx, int ny) { return (nx * ny + 7) / 8; }

// ((ip % n) + n) % n for the ip in [-1, n] reachable from a float angle in [0, 2 pi]; the
// general form only when ip falls outside (it cannot for finite inputs).
__device__ __forceinline__ int wrap_index(int ip, int n) {
    if (ip >= 0 && ip < n) return ip;
    if (ip == -1) return n - 1;
    if (ip == n) return 0;
    return ((ip % n) + n) % n;
}

// nebula3d.py:182-191 shock_field at (i, j, k) (also render.py:165-174 shock_at): max(0, -div v) * rho,
// central differences on clamped neighbours
__device__ __forceinline__ float nb_shock_at(const NbConst& C, const float* __restrict__ rho,
                                             const float* __restrict__ mx, const float* __restrict__ my,
                                             const float* __restrict__ mz, int i, int j, int k) {
    const int nx = C.nx, ny = C.ny, nz = C.nz;
    auto at = [&](const float* a, int ii, int jj, int kk) {
        return __ldg(a + ((long long)iclampd(ii, 0, nx - 1) * ny + iclampd(jj, 0, ny - 1)) * nz + iclampd(kk, 0, nz - 1));
    };
    const float du = at(mx, i + 1, j, k) / at(rho, i + 1, j, k) - at(mx, i - 1, j, k) / at(rho, i - 1, j, k);
    const float dv = at(my, i, j + 1, k) / at(rho, i, j + 1, k) - at(my, i, j - 1, k) / at(rho, i, j - 1, k);
    const float dw = at(mz, i, j, k + 1) / at(rho, i, j, k + 1) - at(mz, i, j, k - 1) / at(rho, i, j, k - 1);
    const float div = (du + dv + dw) / (2.0f * C.dx);
    return fmaxr(-div, 0.0f) * at(rho, i, j, k);
}

// Per-row star constants.  Seen from a star, the cells of one (i, j) row differ only in z: the
// azimuth atan2(ry, rx) of rf_at (nebula3d.py:273-278) / apply_fuv (nebula3d.py:365-368), its
// table column and interpolation weight, and rx^2 + ry^2 are the same for the whole row.  A warp
// (one row) evaluates them once per star, with the same float operations as the per-cell form,
// so every cell sees the same values.  Entry: (rx^2 + ry^2, phi weight, column p0, column p1).
__device__ __forceinline__ void star_row_table(const float4* st, const int* act, int nstars, float px, float py,
                                               int nphi, int colmul, float4* tab) {
    const float two_pi = 2.0f * pi_f();
    for (int s = threadIdx.x; s < nstars; s += 32) {
        if (!act[s]) continue;
        const float4 sp = st[s];
        const float rx = px - sp.x, ry = py - sp.y;
        float phi = atan2f(ry, rx);
        if (phi < 0.0f) phi = phi + two_pi;
        const float fp = phi / two_pi * (float)nphi - 0.5f;
        const int ip = (int)floorf(fp);
        tab[s] = make_float4(rx * rx + ry * ry, fp - (float)ip, __int_as_float(wrap_index(ip, nphi) * colmul),
                             __int_as_float(wrap_index(ip + 1, nphi) * colmul));
    }
    __syncwarp();
}
