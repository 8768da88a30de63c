// Snapshot and frame formats of the simulation state.
//
//  * timeline snapshot (timeline.py:19-89, 13 B/cell): rho, mx, my, mz as fp16 clamped to
//    +-65000, xi as uint8 int(clamp(xi,0,1)*255 + 0.5), dfront / g0 as fp16 (clamped);
//    unpacked back to float32 with rho floored (k_unpack).  One kernel packs every field of a
//    cell (the reference launches one kernel with seven outputs too); the seven output planes
//    live in one caller buffer [rho16 | mx16 | my16 | mz16 | xi8 | df16 | g016].
//  * bake frame (bake.py:95-102, 9 B/cell): g0 = fp16(min(g0, 6e4)), rho = fp16(rho),
//    xi = uint8(round_half_even(clip(xi, 0, 1) * 255)), df = fp16(clip(dfront, -4, 4)),
//    sh = fp16(min(shock, 6e4)) with the shock proxy of nebula3d.py:182-191 computed inline;
//    planes [g016 | rho16 | xi8 | df16 | sh16] in one buffer, so a frame leaves the GPU in one copy.
#include "nb_rayutil.cuh"

namespace {

__device__ __forceinline__ float ld_field(const void* p, long long q, bool half) {
    return half ? __half2float(reinterpret_cast<const __half*>(p)[q]) : reinterpret_cast<const float*>(p)[q];
}

__global__ void __launch_bounds__(256) pack_kernel(const NbConst* __restrict__ c, const float* __restrict__ rho,
                                                   const float* __restrict__ mx, const float* __restrict__ my,
                                                   const float* __restrict__ mz, const float* __restrict__ xi,
                                                   const void* __restrict__ df, const void* __restrict__ g0, bool half,
                                                   unsigned char* __restrict__ out, long long n) {
    const float m = 65000.0f;
    __half* o_r = reinterpret_cast<__half*>(out);
    __half* o_mx = o_r + n;
    __half* o_my = o_mx + n;
    __half* o_mz = o_my + n;
    unsigned char* o_xi = reinterpret_cast<unsigned char*>(o_mz + n);
    __half* o_df = reinterpret_cast<__half*>(o_xi + n);
    __half* o_g0 = o_df + n;
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n; q += (long long)gridDim.x * blockDim.x) {
        o_r[q] = __float2half_rn(fminr(rho[q], m));
        o_mx[q] = __float2half_rn(fminr(fmaxr(-m, mx[q]), m));
        o_my[q] = __float2half_rn(fminr(fmaxr(-m, my[q]), m));
        o_mz[q] = __float2half_rn(fminr(fmaxr(-m, mz[q]), m));
        o_xi[q] = (unsigned char)(int)(fminr(fmaxr(0.0f, xi[q]), 1.0f) * 255.0f + 0.5f);
        o_df[q] = __float2half_rn(fminr(fmaxr(-m, ld_field(df, q, half)), m));
        o_g0[q] = __float2half_rn(fminr(ld_field(g0, q, half), m));
    }
}

__global__ void __launch_bounds__(256) unpack_kernel(const NbConst* __restrict__ c, const unsigned char* __restrict__ in,
                                                     long long n, float* __restrict__ rho, float* __restrict__ mx,
                                                     float* __restrict__ my, float* __restrict__ mz,
                                                     float* __restrict__ xi, void* __restrict__ df,
                                                     void* __restrict__ g0, bool half) {
    const float floor_ = c->floor_;
    const __half* s_r = reinterpret_cast<const __half*>(in);
    const __half* s_mx = s_r + n;
    const __half* s_my = s_mx + n;
    const __half* s_mz = s_my + n;
    const unsigned char* s_xi = reinterpret_cast<const unsigned char*>(s_mz + n);
    const __half* s_df = reinterpret_cast<const __half*>(s_xi + n);
    const __half* s_g0 = s_df + n;
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n; q += (long long)gridDim.x * blockDim.x) {
        rho[q] = fmaxr(__half2float(s_r[q]), floor_);
        mx[q] = __half2float(s_mx[q]);
        my[q] = __half2float(s_my[q]);
        mz[q] = __half2float(s_mz[q]);
        xi[q] = (float)(int)s_xi[q] / 255.0f;
        if (half) {
            reinterpret_cast<__half*>(df)[q] = s_df[q];
            reinterpret_cast<__half*>(g0)[q] = s_g0[q];
        } else {
            reinterpret_cast<float*>(df)[q] = __half2float(s_df[q]);
            reinterpret_cast<float*>(g0)[q] = __half2float(s_g0[q]);
        }
    }
}

__global__ void __launch_bounds__(256) shock_kernel(const NbConst* __restrict__ c, const float* __restrict__ rho,
                                                    const float* __restrict__ mx, const float* __restrict__ my,
                                                    const float* __restrict__ mz, float* __restrict__ out) {
    const NbConst& C = *c;
    const RowWalk w(C.nx, C.ny, C.nz);
    if (!w.valid) return;
    for (int k = w.k0; k < C.nz; k += 32) out[w.base + k] = nb_shock_at(C, rho, mx, my, mz, w.i, w.j, k);
}

__global__ void __launch_bounds__(256) frame_kernel(const NbConst* __restrict__ c, const float* __restrict__ rho,
                                                    const float* __restrict__ mx, const float* __restrict__ my,
                                                    const float* __restrict__ mz, const float* __restrict__ xi,
                                                    const void* __restrict__ df, const void* __restrict__ g0, bool half,
                                                    unsigned char* __restrict__ out, long long n) {
    const NbConst& C = *c;
    const RowWalk w(C.nx, C.ny, C.nz);
    if (!w.valid) return;
    __half* o_g0 = reinterpret_cast<__half*>(out);
    __half* o_r = o_g0 + n;
    unsigned char* o_xi = reinterpret_cast<unsigned char*>(o_r + n);
    __half* o_df = reinterpret_cast<__half*>(o_xi + n);
    __half* o_sh = o_df + n;
    for (int k = w.k0; k < C.nz; k += 32) {
        const long long q = w.base + k;
        const float g = ld_field(g0, q, half);
        // np.minimum(fp16 g0, 6e4) compares in fp16; 6e4 is exact in fp16
        o_g0[q] = __float2half_rn(g < 60000.0f ? g : 60000.0f);
        o_r[q] = __float2half_rn(rho[q]);
        o_xi[q] = (unsigned char)rintf(fminr(fmaxr(0.0f, xi[q]), 1.0f) * 255.0f);
        const float d = ld_field(df, q, half);
        o_df[q] = __float2half_rn(fminr(fmaxr(d, -4.0f), 4.0f));
        const float sh = nb_shock_at(C, rho, mx, my, mz, w.i, w.j, k);
        o_sh[q] = __float2half_rn(sh < 60000.0f ? sh : 60000.0f);
    }
}

int grid_n(long long n) {
    long long b = (n + 255) / 256;
    return (int)(b < 152LL * 16 ? (b < 1 ? 1 : b) : 152LL * 16);
}

}  // namespace

cudaError_t nb_launch_pack(const NbConst* c, const float* rho, const float* mx, const float* my, const float* mz,
                           const float* xi, const void* df, const void* g0, int half, void* out, long long n,
                           cudaStream_t s) {
    pack_kernel<<<grid_n(n), 256, 0, s>>>(c, rho, mx, my, mz, xi, df, g0, half != 0,
                                          static_cast<unsigned char*>(out), n);
    return cudaGetLastError();
}

cudaError_t nb_launch_unpack(const NbConst* c, const void* in, long long n, float* rho, float* mx, float* my,
                             float* mz, float* xi, void* df, void* g0, int half, cudaStream_t s) {
    unpack_kernel<<<grid_n(n), 256, 0, s>>>(c, static_cast<const unsigned char*>(in), n, rho, mx, my, mz, xi, df, g0,
                                            half != 0);
    return cudaGetLastError();
}

cudaError_t nb_launch_shock(const NbConst* c, const float* rho, const float* mx, const float* my, const float* mz,
                            float* out, int nx, int ny, cudaStream_t s) {
    shock_kernel<<<rowwalk_blocks(nx, ny), dim3(32, 8), 0, s>>>(c, rho, mx, my, mz, out);
    return cudaGetLastError();
}

cudaError_t nb_launch_frame(const NbConst* c, const float* rho, const float* mx, const float* my, const float* mz,
                            const float* xi, const void* df, const void* g0, int half, void* out, long long n, int nx,
                            int ny, cudaStream_t s) {
    frame_kernel<<<rowwalk_blocks(nx, ny), dim3(32, 8), 0, s>>>(c, rho, mx, my, mz, xi, df, g0, half != 0,
                                                                static_cast<unsigned char*>(out), n);
    return cudaGetLastError();
}
