// One RK2 stage of the isothermal-Euler update: MUSCL reconstruction (minmod / van Leer /
// MC) + HLL or Rusanov face flux, unsplit x->y->z divergence, wind and jet sources, the
// convex RK combination a*U0 + b*(U + dt*dU), density floor and velocity cap.
//
// Follows nebula3d.py:76-151 (hydro_stage, Rusanov) and sim.py:423-498 (hydro_stage_hll)
// with the face fluxes of nebula3d.py:54-72 / sim.py:397-420.  In the exact build every float
// operation is the reference's, in the reference's order (-fmad=false), so a stage is
// bit-identical to the float32 oracle; the fast build contracts a*b+c, evaluates the fluxes on
// paired FP32 and shares one approximate reciprocal per density.
//
// GB300 layout: a block owns a 32 (k) x TJ (j) column of cells and marches along i over an
// i-chunk.  Each (j,k) plane tile with a 2-cell halo is brought into shared memory by TMA (five
// 3-D tiled loads: rho, mx, my, mz, xi; mbarrier-tracked, bounded waits).  One raw slot: plane
// p+1 is requested as soon as plane p has been converted, and lands while plane p's faces and
// update are computed, which keeps a block at ~56 KB of shared memory and 4 blocks resident per
// SM.  A plane is converted once to primitives (rho, u, v, w) and (c^2, c) in shared memory (each
// thread's own and halo cell, at offsets computed once per tile); every face flux is then
// evaluated once (the reference evaluates each face twice) and shared through shared memory
// (y, z faces; the z faces by warp shuffle where the slopes are kept per cell) or registers (x
// faces; each cell's limited x slope is also carried to the next face).  The exact build also
// evaluates each limited y / z slope once per cell (NB_ONCE_SLOPES).  Sources: the wind loop over the active stars in ionized cells, the jet loop over
// the tile's list of stars whose jet can reach it.  Cell offsets are 32-bit on grids below 2^31
// cells.  Stage 2 also reduces the CFL max speed of the new state (nebula3d.py:154-162) into
// one atomic.
#include <type_traits>

#include "nb_internal.cuh"

namespace {

constexpr int TK = 32;            // cells per tile along k (one warp)
constexpr int RAWW = 40;          // raw tile width along k: [k0-4, k0+36), 16-byte aligned start
constexpr int PW = 36;            // primitive tile width along k: [k0-2, k0+34)

template <int LIM>
__device__ __forceinline__ float slope_lim(float a, float b) {
    if (a * b <= 0.0f) return 0.0f;
    if (LIM == 2) {                                           // sim.py:366-372 mc_lim
        float s = a > 0.0f ? 1.0f : -1.0f;
        return s * fminr(fminr(2.0f * fabsf(a), 2.0f * fabsf(b)), 0.5f * fabsf(a + b));
    }
    if (LIM == 1) return 2.0f * a * b / (a + b);              // sim.py:375-380 vl_lim
    if (fabsf(a) < fabsf(b)) return a;                        // nebula3d.py:40-46 minmod
    return b;
}

#ifndef NB_PAIRED
#if defined(NB_ARITH_FAST) && NB_ARITH_FAST
#define NB_PAIRED 1
#else
#define NB_PAIRED 0
#endif
#endif

// Each limited y / z slope evaluated once per cell and kept in shared memory, or once per face.
// Once per cell pays in the exact build, whose slopes cost a product, two compares and two selects
// per component (stages -5.5%); the fast build's three-operation minmod is cheaper than the extra
// shared-memory traffic (+5% / +8% measured), so it evaluates them per face.  Same bits either way.
#ifndef NB_ONCE_SLOPES
#if NB_PAIRED
#define NB_ONCE_SLOPES 0
#else
#define NB_ONCE_SLOPES 1
#endif
#endif

#if !NB_PAIRED
__device__ __forceinline__ float comp(const float4& v, int c) {
    return c == 0 ? v.x : (c == 1 ? v.y : (c == 2 ? v.z : v.w));
}
#endif

// ---- paired FP32 arithmetic (sm_100+ add/sub/mul/fma.rn.f32x2): a state's four components are
// handled as the pairs (0,1) and (2,3), one instruction issue for two float operations.  Used in
// the fast build only: each paired operation alone rounds as the scalar one, but the assembler
// fuses a dependent mul.rn.f32x2 -> add.rn.f32x2 into one fused multiply-add even with explicit
// round-to-nearest modifiers and -fmad=false (measured on random operands: 13% differ by an ulp),
// which the exact build cannot allow.  The fast build contracts a*b+c anyway.
#if NB_PAIRED
struct F2 {
    unsigned long long v;
};
__device__ __forceinline__ F2 mk2(float a, float b) {
    F2 r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r.v) : "f"(a), "f"(b));
    return r;
}
// one register move unpacks a pair; the unused half is a discarded output of it
#pragma nv_diag_suppress 550
__device__ __forceinline__ float lo(F2 a) {
    float x, y;
    asm("mov.b64 {%0, %1}, %2;" : "=f"(x), "=f"(y) : "l"(a.v));
    return x;
}
__device__ __forceinline__ float hi(F2 a) {
    float x, y;
    asm("mov.b64 {%0, %1}, %2;" : "=f"(x), "=f"(y) : "l"(a.v));
    return y;
}
#pragma nv_diag_default 550
__device__ __forceinline__ F2 add2(F2 a, F2 b) {
    F2 r;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(r.v) : "l"(a.v), "l"(b.v));
    return r;
}
__device__ __forceinline__ F2 sub2(F2 a, F2 b) {
    F2 r;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r.v) : "l"(a.v), "l"(b.v));
    return r;
}
__device__ __forceinline__ F2 mul2(F2 a, F2 b) {
    F2 r;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r.v) : "l"(a.v), "l"(b.v));
    return r;
}
// a*b + c: one fused operation in the fast build, a rounded product then a rounded sum in the exact one
__device__ __forceinline__ F2 madd2(F2 a, F2 b, F2 c) {
#if NB_ARITH_FAST
    F2 r;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r.v) : "l"(a.v), "l"(b.v), "l"(c.v));
    return r;
#else
    return add2(mul2(a, b), c);
#endif
}
// c - a*b with the same rounding rules
__device__ __forceinline__ F2 nmsub2(F2 c, F2 a, F2 b) {
#if NB_ARITH_FAST
    F2 r, na = mk2(-lo(a), -hi(a));
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r.v) : "l"(na.v), "l"(b.v), "l"(c.v));
    return r;
#else
    return sub2(c, mul2(a, b));
#endif
}
__device__ __forceinline__ F2 splat2(float a) { return mk2(a, a); }

// minmod given the product a*b (nebula3d.py:40-46)
__device__ __forceinline__ float minmod_p(float a, float b, float ab) {
    if (ab <= 0.0f) return 0.0f;
    return fabsf(a) < fabsf(b) ? a : b;
}

#if NB_ARITH_FAST
// min.xorsign.abs: min(|a|, |b|) with the sign sign(a) xor sign(b)
__device__ __forceinline__ float min_xorsign(float a, float b) {
    float r;
    asm("min.xorsign.abs.f32 %0, %1, %2;" : "=f"(r) : "f"(a), "f"(b));
    return r;
}
// minmod in three ALU operations and no product: m = min_xorsign(a, b) is min(|a|, |b|) when a and b
// have the same sign, <= 0 otherwise; min_xorsign(a, max(m, 0)) puts a's sign on it.  The value is
// the one minmod_p returns (a or b, the smaller magnitude; ties pick equal values), except that a
// zero result may be -0 (a < 0, or a zero of either sign) where minmod_p returns +0: -0 and +0
// give the same reconstruction b + 0.5 s and c - 0.5 s but for an operand of exactly -0.
__device__ __forceinline__ float minmod_xs(float a, float b) {
    return min_xorsign(a, fmaxf(min_xorsign(a, b), 0.0f));
}
#endif
#endif  // NB_PAIRED

#if NB_ARITH_FAST
// The fast build's reciprocal: one approximate reciprocal (<= 1 ulp) that the three divisions
// by one density share (the exact build divides, as the reference does).
__device__ __forceinline__ float rcp_fast(float x) {
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}
#endif

// Face flux between cells b and c along axis AX (1 = x, 2 = y, 3 = z: the velocity
// component normal to the face).  cs = (c^2, c) of a cell.
//   dot((0, L1, L2, L3), e_AX) == 0 + L_AX exactly (the other products are +-0 and the
//   velocities are finite), and e_c * (rho c^2) == +0 for c != AX.
#if !NB_PAIRED
// The limited slope (4 components) of cell b between its neighbours a and c along one axis:
// slope_lim(b - a, c - b).  A face's right slope is the next face's left slope along the same
// axis (same operands, same bits), which the x march carries from face to face.
template <int LM>
__device__ __forceinline__ float4 slopes_scalar(const float4 qa, const float4 qb, const float4 qc) {
    float sl[4];
#pragma unroll
    for (int c = 0; c < 4; ++c) sl[c] = slope_lim<LM>(comp(qb, c) - comp(qa, c), comp(qc, c) - comp(qb, c));
    return make_float4(sl[0], sl[1], sl[2], sl[3]);
}

// the face flux from the two cells and their limited slopes
template <int SOLVER, int AX>
__device__ __forceinline__ float4 face_flux_scalar_sl(const float4 qb, const float4 qc, const float4 sl,
                                                      const float4 sr, const float2 csb, const float2 csc,
                                                      const float floor_) {
    float L[4], R[4];
#pragma unroll
    for (int c = 0; c < 4; ++c) {
        L[c] = comp(qb, c) + 0.5f * comp(sl, c);
        R[c] = comp(qc, c) - 0.5f * comp(sr, c);
    }
    const float rL = fmaxq(L[0], floor_), rR = fmaxq(R[0], floor_);
    const float unL = 0.0f + L[AX], unR = 0.0f + R[AX];
    const float UL[4] = {rL, rL * L[1], rL * L[2], rL * L[3]};
    const float UR[4] = {rR, rR * R[1], rR * R[2], rR * R[3]};
    const float pL = rL * csb.x, pR = rR * csc.x;
    float FL[4], FR[4], F[4];
#pragma unroll
    for (int c = 0; c < 4; ++c) {
        FL[c] = UL[c] * unL + (c == AX ? pL : 0.0f);
        FR[c] = UR[c] * unR + (c == AX ? pR : 0.0f);
    }
    if (SOLVER == NB_SOLVER_RUSANOV) {
        const float amax = fmaxq(fabsf(unL) + csb.y, fabsf(unR) + csc.y);
        const float ha = 0.5f * amax;
#pragma unroll
        for (int c = 0; c < 4; ++c) F[c] = 0.5f * (FL[c] + FR[c]) - ha * (UR[c] - UL[c]);
        return make_float4(F[0], F[1], F[2], F[3]);
    }
    const float SL = fminq(unL - csb.y, unR - csc.y);
    const float SR = fmaxq(unL + csb.y, unR + csc.y);
    if (SL >= 0.0f) return make_float4(FL[0], FL[1], FL[2], FL[3]);
    if (SR <= 0.0f) return make_float4(FR[0], FR[1], FR[2], FR[3]);
    const float slsr = SL * SR, den = SR - SL;
#pragma unroll
    for (int c = 0; c < 4; ++c) F[c] = (SR * FL[c] - SL * FR[c] + slsr * (UR[c] - UL[c])) / den;
    return make_float4(F[0], F[1], F[2], F[3]);
}

template <int SOLVER, int LIM, int AX>
__device__ __forceinline__ float4 face_flux_scalar(const float4 qa, const float4 qb, const float4 qc, const float4 qd,
                                                   const float2 csb, const float2 csc, const float floor_) {
    constexpr int LM = SOLVER == NB_SOLVER_HLL ? LIM : 0;
    return face_flux_scalar_sl<SOLVER, AX>(qb, qc, slopes_scalar<LM>(qa, qb, qc), slopes_scalar<LM>(qb, qc, qd), csb,
                                           csc, floor_);
}

// The same face flux on component pairs: the float operations and operands of face_flux_scalar
// (the minmod sign test multiplies the same two differences), with a*b+c fused.
#else
// slopes_scalar on component pairs (the minmod sign test multiplies the same two differences)
template <int LM>
__device__ __forceinline__ float4 slopes_paired(const float4 qa, const float4 qb, const float4 qc) {
    const F2 a0 = mk2(qa.x, qa.y), a1 = mk2(qa.z, qa.w), b0 = mk2(qb.x, qb.y), b1 = mk2(qb.z, qb.w);
    const F2 c0 = mk2(qc.x, qc.y), c1 = mk2(qc.z, qc.w);
    const F2 d1_0 = sub2(b0, a0), d1_1 = sub2(b1, a1);
    const F2 d2_0 = sub2(c0, b0), d2_1 = sub2(c1, b1);
    if (LM == 0) {
#if NB_ARITH_FAST
        return make_float4(minmod_xs(lo(d1_0), lo(d2_0)), minmod_xs(hi(d1_0), hi(d2_0)),
                           minmod_xs(lo(d1_1), lo(d2_1)), minmod_xs(hi(d1_1), hi(d2_1)));
#endif
        const F2 p_0 = mul2(d1_0, d2_0), p_1 = mul2(d1_1, d2_1);
        return make_float4(minmod_p(lo(d1_0), lo(d2_0), lo(p_0)), minmod_p(hi(d1_0), hi(d2_0), hi(p_0)),
                           minmod_p(lo(d1_1), lo(d2_1), lo(p_1)), minmod_p(hi(d1_1), hi(d2_1), hi(p_1)));
    }
    return make_float4(slope_lim<LM>(lo(d1_0), lo(d2_0)), slope_lim<LM>(hi(d1_0), hi(d2_0)),
                       slope_lim<LM>(lo(d1_1), lo(d2_1)), slope_lim<LM>(hi(d1_1), hi(d2_1)));
}

// The same face flux on component pairs: the float operations and operands of face_flux_scalar_sl,
// with a*b+c fused.
template <int SOLVER, int AX>
__device__ __forceinline__ float4 face_flux_paired_sl(const float4 qb, const float4 qc, const float4 sl,
                                                      const float4 sr, const float2 csb, const float2 csc,
                                                      const float floor_) {
    const F2 b0 = mk2(qb.x, qb.y), b1 = mk2(qb.z, qb.w), c0 = mk2(qc.x, qc.y), c1 = mk2(qc.z, qc.w);
    const F2 sl0 = mk2(sl.x, sl.y), sl1 = mk2(sl.z, sl.w), sr0 = mk2(sr.x, sr.y), sr1 = mk2(sr.z, sr.w);
    const F2 half = splat2(0.5f);
    const F2 L0 = madd2(half, sl0, b0), L1 = madd2(half, sl1, b1);      // b + 0.5 * slope
    const F2 R0 = nmsub2(c0, half, sr0), R1 = nmsub2(c1, half, sr1);    // c - 0.5 * slope
    const float rL = fmaxq(lo(L0), floor_), rR = fmaxq(lo(R0), floor_);
    const float unL = 0.0f + (AX == 1 ? hi(L0) : (AX == 2 ? lo(L1) : hi(L1)));
    const float unR = 0.0f + (AX == 1 ? hi(R0) : (AX == 2 ? lo(R1) : hi(R1)));
    // U = (r, r u, r v, r w): r * 1 == r exactly
    const F2 UL0 = mul2(splat2(rL), mk2(1.0f, hi(L0))), UL1 = mul2(splat2(rL), L1);
    const F2 UR0 = mul2(splat2(rR), mk2(1.0f, hi(R0))), UR1 = mul2(splat2(rR), R1);
    const float pL = rL * csb.x, pR = rR * csc.x;
    // F = U * un + p e_AX (the other components add +0, as the reference's e_c * p does)
    const F2 pL0 = mk2(0.0f, AX == 1 ? pL : 0.0f), pL1 = mk2(AX == 2 ? pL : 0.0f, AX == 3 ? pL : 0.0f);
    const F2 pR0 = mk2(0.0f, AX == 1 ? pR : 0.0f), pR1 = mk2(AX == 2 ? pR : 0.0f, AX == 3 ? pR : 0.0f);
    const F2 FL0 = madd2(UL0, splat2(unL), pL0), FL1 = madd2(UL1, splat2(unL), pL1);
    const F2 FR0 = madd2(UR0, splat2(unR), pR0), FR1 = madd2(UR1, splat2(unR), pR1);
    if (SOLVER == NB_SOLVER_RUSANOV) {
        const float amax = fmaxq(fabsf(unL) + csb.y, fabsf(unR) + csc.y);
        const F2 ha = splat2(0.5f * amax);
        const F2 F0 = nmsub2(mul2(half, add2(FL0, FR0)), ha, sub2(UR0, UL0));
        const F2 F1 = nmsub2(mul2(half, add2(FL1, FR1)), ha, sub2(UR1, UL1));
        return make_float4(lo(F0), hi(F0), lo(F1), hi(F1));
    }
#if NB_ARITH_FAST
    // branch-free: min(SL, 0) and max(SR, 0) in the general formula give FL (SL >= 0) and FR
    // (SR <= 0) up to the rounding of SR FL / SR; SR - SL >= 2 c > 0 keeps the denominator positive
    const float SL = fminf(fminq(unL - csb.y, unR - csc.y), 0.0f);
    const float SR = fmaxf(fmaxq(unL + csb.y, unR + csc.y), 0.0f);
#else
    const float SL = fminq(unL - csb.y, unR - csc.y);
    const float SR = fmaxq(unL + csb.y, unR + csc.y);
    if (SL >= 0.0f) return make_float4(lo(FL0), hi(FL0), lo(FL1), hi(FL1));
    if (SR <= 0.0f) return make_float4(lo(FR0), hi(FR0), lo(FR1), hi(FR1));
#endif
    const F2 slsr = splat2(SL * SR);
    const float den = SR - SL;
    // (SR FL - SL FR + SL SR (UR - UL)) / den, every product feeding a sum as an explicit fused
    // multiply-add (a paired multiply followed by a paired add would be fused or not at the
    // assembler's discretion, which could differ between the single and the batched kernel)
    const F2 nSL = splat2(-SL), SR2 = splat2(SR);
    const F2 T0 = madd2(slsr, sub2(UR0, UL0), madd2(SR2, FL0, mul2(nSL, FR0)));
    const F2 T1 = madd2(slsr, sub2(UR1, UL1), madd2(SR2, FL1, mul2(nSL, FR1)));
#if NB_ARITH_FAST
    const F2 inv = splat2(rcp_fast(den));
    const F2 F0 = mul2(T0, inv), F1 = mul2(T1, inv);
    return make_float4(lo(F0), hi(F0), lo(F1), hi(F1));
#else
    return make_float4(lo(T0) / den, hi(T0) / den, lo(T1) / den, hi(T1) / den);
#endif
}

template <int SOLVER, int LIM, int AX>
__device__ __forceinline__ float4 face_flux_paired(const float4 qa, const float4 qb, const float4 qc, const float4 qd,
                                                   const float2 csb, const float2 csc, const float floor_) {
    constexpr int LM = SOLVER == NB_SOLVER_HLL ? LIM : 0;
    return face_flux_paired_sl<SOLVER, AX>(qb, qc, slopes_paired<LM>(qa, qb, qc), slopes_paired<LM>(qb, qc, qd), csb,
                                           csc, floor_);
}
#endif  // NB_PAIRED

template <int SOLVER, int LIM, int AX>
__device__ __forceinline__ float4 face_flux(const float4 qa, const float4 qb, const float4 qc, const float4 qd,
                                            const float2 csb, const float2 csc, const float floor_) {
#if NB_PAIRED
    return face_flux_paired<SOLVER, LIM, AX>(qa, qb, qc, qd, csb, csc, floor_);
#else
    return face_flux_scalar<SOLVER, LIM, AX>(qa, qb, qc, qd, csb, csc, floor_);
#endif
}

// the face flux from the face's two cells and their limited slopes along its axis
template <int SOLVER, int AX>
__device__ __forceinline__ float4 face_flux_sl(const float4 qb, const float4 qc, const float4 sl, const float4 sr,
                                               const float2 csb, const float2 csc, const float floor_) {
#if NB_PAIRED
    return face_flux_paired_sl<SOLVER, AX>(qb, qc, sl, sr, csb, csc, floor_);
#else
    return face_flux_scalar_sl<SOLVER, AX>(qb, qc, sl, sr, csb, csc, floor_);
#endif
}

template <int SOLVER, int LIM>
__device__ __forceinline__ float4 cell_slopes(const float4 qa, const float4 qb, const float4 qc) {
    constexpr int LM = SOLVER == NB_SOLVER_HLL ? LIM : 0;
#if NB_PAIRED
    return slopes_paired<LM>(qa, qb, qc);
#else
    return slopes_scalar<LM>(qa, qb, qc);
#endif
}

// The x face between cells b and c of the march: `slope` holds cell b's limited slope on entry
// (the previous face's right slope) and cell c's on return.
template <int SOLVER, int LIM>
__device__ __forceinline__ float4 face_flux_x(const float4 qb, const float4 qc, const float4 qd, const float2 csb,
                                              const float2 csc, const float floor_, float4& slope) {
    const float4 sl = slope;
    slope = cell_slopes<SOLVER, LIM>(qb, qc, qd);
#if NB_PAIRED
    return face_flux_paired_sl<SOLVER, 1>(qb, qc, sl, slope, csb, csc, floor_);
#else
    return face_flux_scalar_sl<SOLVER, 1>(qb, qc, sl, slope, csb, csc, floor_);
#endif
}

template <int TJ>
struct HydroSmem {
    static constexpr int RAW_FIELD = (TJ + 4) * RAWW;                     // floats per field
    static constexpr int RAW_BYTES = 5 * RAW_FIELD * 4;                      // one raw slot
#if NB_ONCE_SLOPES
    static constexpr int PRIM_BYTES = 3 * (TJ + 4) * PW * 16;               // planes p-2, p-1, p
    static constexpr int CS_BYTES = 3 * (TJ + 4) * PW * 8;
    static constexpr int SY_BYTES = (TJ + 2) * TK * 16;                     // y slopes, rows j0-1 .. j0+TJ
    static constexpr int SZ_BYTES = TJ * (TK + 2) * 16;                     // z slopes, columns k0-1 .. k0+TK
    static constexpr int FACE_BYTES = ((TJ + 1) * TK + TJ) * 16;            // y faces; the z faces k0-1/2
#else
    static constexpr int PRIM_BYTES = 4 * (TJ + 4) * PW * 16;               // planes p-3 .. p
    static constexpr int CS_BYTES = 3 * (TJ + 4) * PW * 8;
    static constexpr int SY_BYTES = 0, SZ_BYTES = 0;
    static constexpr int FACE_BYTES = ((TJ + 1) * TK + TJ * (TK + 1)) * 16; // y faces; z faces
#endif
    static constexpr int BAR_BYTES = 64;
    static constexpr int FIXED = RAW_BYTES + PRIM_BYTES + CS_BYTES + SY_BYTES + SZ_BYTES + FACE_BYTES + BAR_BYTES;
    // star tables: positions / wind weights and jets (2 x float4 per star), then the tile's jet
    // list: a count and the indices (one byte each) of the stars whose jet can reach the tile
    __host__ __device__ static int jet_list_offset(int nstars) { return FIXED + nstars * 32; }
    static int bytes(int nstars) { return jet_list_offset(nstars) + 16 + ((nstars + 15) & ~15); }
};

#ifndef NB_HYDRO_TJ
#define NB_HYDRO_TJ 8                 // tile rows along j (one warp per row; 16 measured 2% slower; hydro_tile assumes 8)
#endif
#ifndef NB_HYDRO_MINB
#define NB_HYDRO_MINB (32 / NB_HYDRO_TJ)  // resident blocks per SM the register budget is sized for (64 regs)
#endif

// One (j,k) tile column of one instance, marched over its i-chunk.  Called once per block by
// the single-instance kernel and once per work item by the persistent batched kernel.  The
// two mbarriers and their phases persist across calls: every load a call issues, it waits for.
// `rot` (0-3, the same in every thread of the block) spreads the per-plane work that only some
// warps do -- the y faces below the tile, the z faces before it, the z-halo conversion and the TMA
// issue -- over warps of four different schedulers (warp w is issued by scheduler w mod 4 when a
// block's warp slots start at a multiple of 4), rotated from block to block; any value gives the
// same results.
template <int SOLVER, int LIM, int TJ, bool STAGE2, bool I32 = false>
__device__ __forceinline__ void hydro_tile(const HydroLaunch& L, int tile, unsigned char* smem, unsigned& ph0,
                                           bool& failed, int rot) {
    static_assert(TJ == 8, "the halo and edge-face warp assignment assumes 8 warps of 32 threads");
    using Idx = typename std::conditional<I32, int, long long>::type;     // the own cell's offset
    using SM = HydroSmem<TJ>;
    {
        // an opaque zero added to the shared-memory base: the compiler then derives the tiles'
        // addresses from one register rather than holding several precomputed bases (measured at
        // 256^3: stage spills 4 -> 0 bytes, stages -3%, the same code otherwise)
        unsigned zero = 0;
        asm volatile("" : "+r"(zero));
        smem += zero;
    }
    float* raw = reinterpret_cast<float*>(smem);                                   // [5][TJ+4][40]
    float4* prim = reinterpret_cast<float4*>(smem + SM::RAW_BYTES);                // [4 or 3][TJ+4][36]
    float2* cs = reinterpret_cast<float2*>(smem + SM::RAW_BYTES + SM::PRIM_BYTES); // [3][TJ+4][36]
#if NB_ONCE_SLOPES
    float4* sy = reinterpret_cast<float4*>(smem + SM::RAW_BYTES + SM::PRIM_BYTES + SM::CS_BYTES);  // [TJ+2][32]
    float4* sz = sy + (TJ + 2) * TK;                                               // [TJ][34]
    float4* fy = sz + TJ * (TK + 2);                                               // [TJ+1][32]
    float4* fz0 = fy + (TJ + 1) * TK;                                              // [TJ]
#else
    float4* fy = reinterpret_cast<float4*>(smem + SM::RAW_BYTES + SM::PRIM_BYTES + SM::CS_BYTES);  // [TJ+1][32]
    float4* fz = fy + (TJ + 1) * TK;                                               // [TJ][33]
#endif
    uint64_t* bar = reinterpret_cast<uint64_t*>(smem + SM::FIXED - SM::BAR_BYTES);
    float4* sw_w = reinterpret_cast<float4*>(smem + SM::FIXED);
    const NbConst& C = *L.c;
    const int nx = C.nx, ny = C.ny, nz = C.nz, nstars = L.no_sources ? 0 : C.nstars;
    float4* sw_j = sw_w + nstars;

    const int tid = threadIdx.x, tk = tid & 31, tj = tid >> 5;
    int kt, jt, ci;
    if (L.order == 0) {                       // sweep order 0: k tiles fastest, then j, then i-chunks
        kt = tile % L.tiles_k;
        tile /= L.tiles_k;
        jt = tile % L.tiles_j;
        ci = tile / L.tiles_j;
    } else {                                  // sweep order 1: i-chunks fastest, then k, then j
        ci = tile % L.n_chunks;
        tile /= L.n_chunks;
        kt = tile % L.tiles_k;
        jt = tile / L.tiles_k;
    }
    const int k0 = kt * TK, j0 = jt * TJ;
    // n_chunks = ceil(nx / chunk_i) chunks of equal depth (within one plane): no short last chunk
    const int i0 = (int)((long long)ci * nx / L.n_chunks);
    const int i_end = (int)((long long)(ci + 1) * nx / L.n_chunks);
    const int P0 = i0 - 2, P1 = i_end + 1;

    const float floor_ = C.floor_, cn2 = C.cn2, ci2 = C.ci2, vmax = C.vmax, dx = C.dx;
    const float dt = L.use_override ? L.dt_override : L.st->dt_f;
    const float pulse = L.use_override ? L.pulse_override : L.st->pulse_f;
    const float wind = L.no_sources ? 0.0f : C.wind_f, jet_cos = C.jet_cos_f, jet_r = C.jet_r_f;
    const float a = L.a, b = L.b;

    int* n_jet_p = reinterpret_cast<int*>(smem + SM::jet_list_offset(nstars));
    unsigned char* jet_ix = smem + SM::jet_list_offset(nstars) + 16;
    for (int s = tid; s < nstars; s += blockDim.x) {
        sw_w[s] = L.sw[s].w;
        sw_j[s] = L.sw[s].jet;
    }
    constexpr unsigned TX_BYTES = 5u * SM::RAW_FIELD * 4u;
    auto issue = [&](int p) {                    // plane p into the raw slot, tracked by bar[0]
        if (!L.maps) return;                     // failure-path test: the wait for it runs out
        const int pc = iclampd(p, 0, nx - 1);
        fence_proxy_async();                     // the slot's previous contents were read by this block
        mbar_expect_tx(&bar[0], TX_BYTES);
#pragma unroll
        for (int f = 0; f < 4; ++f)
            tma_load_3d(raw + f * SM::RAW_FIELD, &L.maps[L.map_in + f], k0 - 4, j0 - 2, pc, &bar[0]);
        tma_load_3d(raw + 4 * SM::RAW_FIELD, &L.maps[NB_MAP_XI], k0 - 4, j0 - 2, pc, &bar[0]);
    };
    // the per-plane extra work, on warps of schedulers rot, rot+1, rot+2 and rot+3 (mod 4): the y
    // faces below the tile (role bit 1), the z faces before it (bit 2), the z-halo conversion,
    // the TMA issue (bit 4); with once-per-cell slopes also the slopes of the halo cells the faces
    // read: the y slopes of row j0-1 (bit 8) and of row j0+TJ (bit 16), the z slopes of columns
    // k0-1 and k0+TK (bit 32)
    const int w_zhalo = 4 + ((rot + 2) & 3);
    const unsigned role = (tj == rot ? 1u : 0u) | (tj == ((rot + 1) & 3) && tk < TJ ? 2u : 0u) |
                          (tid == (4 + ((rot + 3) & 3)) * 32 ? 4u : 0u) |
                          (NB_ONCE_SLOPES && tj == 4 + (rot & 3) ? 8u : 0u) |
                          (NB_ONCE_SLOPES && tj == 4 + ((rot + 1) & 3) ? 16u : 0u) |
                          (NB_ONCE_SLOPES && tj == 4 + ((rot + 3) & 3) && tk < 2 * TJ ? 32u : 0u);
    if (role & 4u) issue(P0);
    if (tj == 0) {
        // The stars whose jet (nebula3d.py:131-149: strength > 0, an active star, r < jet_r) can reach
        // a cell centre of this tile, in star order: the distance from the star to the box of the
        // tile's cell centres, less a margin of two cells for the float rounding of the per-cell
        // distance, must be below jet_r.  Stars left out add exactly nothing to any cell here.
        const float bx0 = ((float)i0 + 0.5f) * dx, bx1 = ((float)(i_end - 1) + 0.5f) * dx;
        const float by0 = ((float)j0 + 0.5f) * dx, by1 = ((float)(min(j0 + TJ, ny) - 1) + 0.5f) * dx;
        const float bz0 = ((float)k0 + 0.5f) * dx, bz1 = ((float)(min(k0 + TK, nz) - 1) + 0.5f) * dx;
        const float reach = jet_r + 2.0f * dx;
        int n = 0;
        for (int s0 = 0; s0 < nstars; s0 += 32) {
            const int s = s0 + tk;
            bool keep = false;
            if (s < nstars) {
                const float4 st = L.sw[s].w, jt = L.sw[s].jet;
                if (jt.w > 0.0f && st.w > 0.0f) {
                    const float ex = fmaxf(0.0f, fmaxf(bx0 - st.x, st.x - bx1));
                    const float ey = fmaxf(0.0f, fmaxf(by0 - st.y, st.y - by1));
                    const float ez = fmaxf(0.0f, fmaxf(bz0 - st.z, st.z - bz1));
                    keep = !(ex * ex + ey * ey + ez * ez >= reach * reach);    // NaN keeps the star
                }
            }
            const unsigned m = __ballot_sync(0xffffffffu, keep);
            if (keep) jet_ix[n + __popc(m & ((1u << tk) - 1u))] = (unsigned char)s;
            n += __popc(m);
        }
        if (tk == 0) *n_jet_p = n;
    }

    float4 fx_prev = make_float4(0.f, 0.f, 0.f, 0.f);
    float4 xslope = make_float4(0.f, 0.f, 0.f, 0.f);    // limited x slope of the march's cell p-2
    float vmax_local = 0.0f;

    // clamped global -> raw-tile coordinates
    auto raw_at = [&](int jj, int kk) {      // jj, kk: prim-tile coords
        const int jc = iclampd(j0 - 2 + jj, 0, ny - 1) - (j0 - 2);
        const int kc = iclampd(k0 - 2 + kk, 0, nz - 1) - (k0 - 4);
        return jc * RAWW + kc;
    };
    const int own = (tj + 2) * PW + tk + 2;          // this thread's cell in a prim / cs tile
    // the cells this thread converts in every plane: its own, and one of the 4 TK + 4 TJ cells of
    // the halo strips (corners are never read): warps 0-3 one row of the y strips each, warp
    // w_zhalo the z strips; their offsets, computed once per tile, clamp to the domain in the raw tile
    const bool has_halo = tj < 4 || tj == w_zhalo;
    const int raw_own = raw_at(tj + 2, tk + 2);
    int prim_halo = 0, raw_halo = 0;
    if (has_halo) {
        int jj, kk;
        if (tj < 4) {
            jj = tj < 2 ? tj : TJ + tj;
            kk = 2 + tk;
        } else {
            const int hh = tk;
            jj = 2 + (hh >> 2);
            const int q = hh & 3;
            kk = q < 2 ? q : 32 + q;
        }
        prim_halo = jj * PW + kk;
        raw_halo = raw_at(jj, kk);
    }
    const int j = j0 + tj, k = k0 + tk;
    const bool inside = j < ny && k < nz;
    constexpr int PSLOT = (TJ + 4) * PW;

    for (int p = P0; p <= P1; ++p) {
#if NB_ONCE_SLOPES
        // slots of planes p, p-1, p-2 in the three-plane rings of primitives and sound speeds
        const int cq = (p - P0) % 3;
        const int cq1 = cq == 0 ? 2 : cq - 1;
        const int cq2 = cq1 == 0 ? 2 : cq1 - 1;
        const int ps = cq;
#else
        const int ps = (p - P0) & 3;                 // prim slot of plane p (4 slots: p-3..p)
        const int cq = (p - P0) % 3;                 // cs slot of plane p (3 slots: p-2..p)
#endif
        // own-cell values of plane i = p - 2 the epilogue needs, issued before the flux work
        const int i = p - 2;
        const Idx cell = ((Idx)i * ny + j) * nz + k;
        const bool work = p >= i0 + 2;
        float u00 = 0.f, u01 = 0.f, u02 = 0.f, u03 = 0.f, ur = 0.f, umx = 0.f, umy = 0.f, umz = 0.f, uxi = 0.f;
        if (work && inside) {
            ur = L.in[0][cell]; umx = L.in[1][cell]; umy = L.in[2][cell]; umz = L.in[3][cell];
            uxi = L.xi[cell];
            if (STAGE2) {                        // early: read only at the end, 4 more live registers
                u00 = L.u0[0][cell]; u01 = L.u0[1][cell]; u02 = L.u0[2][cell]; u03 = L.u0[3][cell];
            }
        }
        const int jj = tj + 2, kk = tk + 2;
#if NB_ONCE_SLOPES
        if (work) {
            // ---- the limited y and z slopes of every cell of plane i that the faces read, each
            // evaluated once (a face's two slopes are its cells' slopes along its axis: the same
            // operands, the same bits).  Plane i was converted two planes ago and the previous
            // plane's faces are done (its second barrier), so no barrier is needed here, and this
            // work overlaps the wait for plane p's tile.
            const float4* q = prim + cq2 * PSLOT;
            const float4 qo = q[jj * PW + kk];
            sy[(tj + 1) * TK + tk] = cell_slopes<SOLVER, LIM>(q[(jj - 1) * PW + kk], qo, q[(jj + 1) * PW + kk]);
            sz[tj * (TK + 2) + tk + 1] = cell_slopes<SOLVER, LIM>(q[jj * PW + kk - 1], qo, q[jj * PW + kk + 1]);
            if (role & 8u)                       // row j0-1: primitive rows 0..2
                sy[tk] = cell_slopes<SOLVER, LIM>(q[0 * PW + kk], q[1 * PW + kk], q[2 * PW + kk]);
            if (role & 16u)                      // row j0+TJ: primitive rows TJ+1..TJ+3
                sy[(TJ + 1) * TK + tk] = cell_slopes<SOLVER, LIM>(q[(TJ + 1) * PW + kk], q[(TJ + 2) * PW + kk],
                                                                  q[(TJ + 3) * PW + kk]);
            if (role & 32u) {                    // columns k0-1 (lanes 0..TJ-1) and k0+TK (lanes TJ..2TJ-1)
                const int r = tk & (TJ - 1);
                const int c0 = tk < TJ ? 0 : TK + 1;
                const int b = (r + 2) * PW + c0;
                sz[r * (TK + 2) + c0] = cell_slopes<SOLVER, LIM>(q[b], q[b + 1], q[b + 2]);
            }
        }
#endif
        const bool ok = mbar_wait_limited(&bar[0], ph0, &L.wait_limit);
        if (ok) ph0 ^= 1u;                       // a timed-out wait keeps its parity for the abort wait
        if (__syncthreads_or(!ok)) { failed = true; break; }
        const float* rb = raw;
        float4* pp = prim + ps * PSLOT;
        float2* cp = cs + cq * PSLOT;
        // ---- convert plane p: the own cell, then (has_halo) one cell of the halo strips
        auto convert = [&](int o, int pi) {
            const float r = fmaxq(rb[o], floor_);
            const float xv = rb[4 * SM::RAW_FIELD + o];
            const float c2 = cn2 + xv * (ci2 - cn2);
#if NB_ARITH_FAST
            const float ri = rcp_fast(r);
            pp[pi] = make_float4(r, rb[SM::RAW_FIELD + o] * ri, rb[2 * SM::RAW_FIELD + o] * ri,
                                 rb[3 * SM::RAW_FIELD + o] * ri);
#else
            pp[pi] = make_float4(r, rb[SM::RAW_FIELD + o] / r, rb[2 * SM::RAW_FIELD + o] / r,
                                 rb[3 * SM::RAW_FIELD + o] / r);
#endif
            cp[pi] = make_float2(c2, sqrtf(c2));
        };
        convert(raw_own, own);
        if (has_halo) convert(raw_halo, prim_halo);
        __syncthreads();                         // every thread is done with the raw slot
        if ((role & 4u) && p + 1 <= P1) issue(p + 1);
#if NB_ONCE_SLOPES
        if (p < P0 + 2) continue;
        if (p == P0 + 2) {                       // the x slope of plane P0+1 (planes P0, P0+1, P0+2)
            xslope = cell_slopes<SOLVER, LIM>(prim[cq2 * PSLOT + own], prim[cq1 * PSLOT + own], pp[own]);
            continue;
        }
        // x face (p-2)+1/2 from the own column of planes p-2..p and the carried slope of p-2
        const float4 fx_new = face_flux_x<SOLVER, LIM>(prim[cq2 * PSLOT + own], prim[cq1 * PSLOT + own], pp[own],
                                                       cs[cq2 * PSLOT + own], cs[cq1 * PSLOT + own], floor_, xslope);
        if (!work) { fx_prev = fx_new; continue; }
        // ---- the y and z faces of cell plane i, from the cells and their slopes
        const float4* q = prim + cq2 * PSLOT;
        const float2* c = cs + cq2 * PSLOT;
        const float4 fyp = face_flux_sl<SOLVER, 2>(q[jj * PW + kk], q[(jj + 1) * PW + kk], sy[(tj + 1) * TK + tk],
                                                   sy[(tj + 2) * TK + tk], c[jj * PW + kk], c[(jj + 1) * PW + kk],
                                                   floor_);
        const float4 fzp = face_flux_sl<SOLVER, 3>(q[jj * PW + kk], q[jj * PW + kk + 1], sz[tj * (TK + 2) + tk + 1],
                                                   sz[tj * (TK + 2) + tk + 2], c[jj * PW + kk], c[jj * PW + kk + 1],
                                                   floor_);
        fy[(tj + 1) * TK + tk] = fyp;
        if (role & 1u) {                        // the y face below the tile: (j0-1)+1/2
            fy[tk] = face_flux_sl<SOLVER, 2>(q[1 * PW + kk], q[2 * PW + kk], sy[tk], sy[TK + tk], c[1 * PW + kk],
                                             c[2 * PW + kk], floor_);
        } else if (role & 2u) {                 // the z face before the tile in row tk: (k0-1)+1/2
            const int r2 = (tk + 2) * PW;
            fz0[tk] = face_flux_sl<SOLVER, 3>(q[r2 + 1], q[r2 + 2], sz[tk * (TK + 2)], sz[tk * (TK + 2) + 1],
                                              c[r2 + 1], c[r2 + 2], floor_);
        }
        __syncthreads();
        const float4 fym = fy[tj * TK + tk];
        // the z face k-1/2 is the lower lane's k+1/2; lane 0 takes the face before the tile
        float4 fzm = make_float4(__shfl_up_sync(0xffffffffu, fzp.x, 1), __shfl_up_sync(0xffffffffu, fzp.y, 1),
                                 __shfl_up_sync(0xffffffffu, fzp.z, 1), __shfl_up_sync(0xffffffffu, fzp.w, 1));
        if (tk == 0) fzm = fz0[tj];
#else
        if (p < P0 + 3) continue;
        // x face (p-2)+1/2 from the own column of planes p-2..p and the carried slope of p-2
        const float4 qx1 = prim[((p - 2 - P0) & 3) * PSLOT + own], qx2 = prim[((p - 1 - P0) & 3) * PSLOT + own];
        if (p == P0 + 3) xslope = cell_slopes<SOLVER, LIM>(prim[((p - 3 - P0) & 3) * PSLOT + own], qx1, qx2);
        const float4 fx_new = face_flux_x<SOLVER, LIM>(qx1, qx2, pp[own], cs[((p - 2 - P0) % 3) * PSLOT + own],
                                                       cs[((p - 1 - P0) % 3) * PSLOT + own], floor_, xslope);
        if (!work) { fx_prev = fx_new; continue; }
        // ---- cell plane i = p - 2
        const int si = (i - P0) & 3;
        const float4* q = prim + si * PSLOT;
        const float2* c = cs + ((i - P0) % 3) * PSLOT;
        const float4 fyp = face_flux<SOLVER, LIM, 2>(q[(jj - 1) * PW + kk], q[jj * PW + kk], q[(jj + 1) * PW + kk],
                                                     q[(jj + 2) * PW + kk], c[jj * PW + kk], c[(jj + 1) * PW + kk],
                                                     floor_);
        const float4 fzp = face_flux<SOLVER, LIM, 3>(q[jj * PW + kk - 1], q[jj * PW + kk], q[jj * PW + kk + 1],
                                                     q[jj * PW + kk + 2], c[jj * PW + kk], c[jj * PW + kk + 1],
                                                     floor_);
        fy[(tj + 1) * TK + tk] = fyp;
        fz[tj * (TK + 1) + tk + 1] = fzp;
        if (role & 1u) {                        // the y face below the tile: (j0-1)+1/2
            fy[tk] = face_flux<SOLVER, LIM, 2>(q[0 * PW + kk], q[1 * PW + kk], q[2 * PW + kk], q[3 * PW + kk],
                                               c[1 * PW + kk], c[2 * PW + kk], floor_);
        } else if (role & 2u) {                 // the z face before the tile in row tk: (k0-1)+1/2
            const int r2 = (tk + 2) * PW;
            fz[tk * (TK + 1)] = face_flux<SOLVER, LIM, 3>(q[r2 + 0], q[r2 + 1], q[r2 + 2], q[r2 + 3], c[r2 + 1],
                                                          c[r2 + 2], floor_);
        }
        __syncthreads();
        const float4 fym = fy[tj * TK + tk];
        const float4 fzm = fz[tj * (TK + 1) + tk];
#endif
        const float4 fxp = fx_new, fxm = fx_prev;
        fx_prev = fx_new;
        // div = 0 + (fR-fL)_x, then += (fR-fL)_y, then += (fR-fL)_z  (nebula3d.py:87-109)
        float du0, du1, du2, du3;
#if NB_PAIRED
        {
            const F2 dA = add2(add2(sub2(mk2(fxp.x, fxp.y), mk2(fxm.x, fxm.y)), sub2(mk2(fyp.x, fyp.y), mk2(fym.x, fym.y))),
                               sub2(mk2(fzp.x, fzp.y), mk2(fzm.x, fzm.y)));
            const F2 dB = add2(add2(sub2(mk2(fxp.z, fxp.w), mk2(fxm.z, fxm.w)), sub2(mk2(fyp.z, fyp.w), mk2(fym.z, fym.w))),
                               sub2(mk2(fzp.z, fzp.w), mk2(fzm.z, fzm.w)));
            const F2 sc = splat2(C.dx_pow2 ? -C.inv_dx : -1.0f / dx);
            const F2 uA = mul2(dA, sc), uB = mul2(dB, sc);
            du0 = lo(uA); du1 = hi(uA); du2 = lo(uB); du3 = hi(uB);
        }
#else
        float d0 = 0.0f + (fxp.x - fxm.x), d1 = 0.0f + (fxp.y - fxm.y);
        float d2 = 0.0f + (fxp.z - fxm.z), d3 = 0.0f + (fxp.w - fxm.w);
        d0 = d0 + (fyp.x - fym.x); d1 = d1 + (fyp.y - fym.y); d2 = d2 + (fyp.z - fym.z); d3 = d3 + (fyp.w - fym.w);
        d0 = d0 + (fzp.x - fzm.x); d1 = d1 + (fzp.y - fzm.y); d2 = d2 + (fzp.z - fzm.z); d3 = d3 + (fzp.w - fzm.w);
        // ---- sources and RK combination (nebula3d.py:111-151)
        if (C.dx_pow2) {
            const float sc = C.inv_dx;
            du0 = -d0 * sc; du1 = -d1 * sc; du2 = -d2 * sc; du3 = -d3 * sc;
        } else {
            du0 = -d0 / dx; du1 = -d1 / dx; du2 = -d2 / dx; du3 = -d3 / dx;
        }
#endif
        const float px = ((float)i + 0.5f) * dx, py = ((float)j + 0.5f) * dx, pz = ((float)k + 0.5f) * dx;
        const float x_ion = uxi;
        if (wind > 0.0f && x_ion > 0.01f) {
            float ax = 0.0f, ay = 0.0f, az = 0.0f;
            for (int s = 0; s < nstars; ++s) {
                const float4 st = sw_w[s];
                if (st.w > 0.0f) {
                    const float rx = px - st.x, ry = py - st.y, rz = pz - st.z;
                    const float r2 = ((rx * rx + ry * ry) + rz * rz) + 0.0004f;     // 0 + x*x == x*x
                    const float f = st.w / (r2 * sqrtf(r2));
                    ax = ax + rx * f; ay = ay + ry * f; az = az + rz * f;
                }
            }
            const float wx = wind * x_ion;
            ax = ax * wx; ay = ay * wx; az = az * wx;
            du0 = du0 + 0.0f;
            du1 = du1 + ur * ax; du2 = du2 + ur * ay; du3 = du3 + ur * az;
        }
        float jx = 0.0f, jy = 0.0f, jz = 0.0f;
        const int n_jet = *n_jet_p;
        for (int m = 0; m < n_jet; ++m) {
            const int s = jet_ix[m];
            const float4 jt = sw_j[s];
            const float4 st = sw_w[s];
            {
                const float rx = px - st.x, ry = py - st.y, rz = pz - st.z;
                const float r = sqrtf((rx * rx + ry * ry) + rz * rz);
                if (r < jet_r && r > 1e-6f) {
                    const float cth = (((0.0f + rx * jt.x) + ry * jt.y) + rz * jt.z) / r;
                    if (fabsf(cth) > jet_cos) {
                        const float f = (cth > 0.0f ? 1.0f : -1.0f) * jt.w * pulse / (r * r + 0.0004f);
                        jx = jx + jt.x * f; jy = jy + jt.y * f; jz = jz + jt.z * f;
                    }
                }
            }
        }
        du0 = du0 + 0.0f;
        du1 = du1 + ur * jx; du2 = du2 + ur * jy; du3 = du3 + ur * jz;
        if (!STAGE2) {
            u00 = ur; u01 = umx; u02 = umy; u03 = umz;
        }
#if NB_PAIRED
        float o0, o1, o2, o3;
        {
            const F2 dt2 = splat2(dt);
            const F2 nA = madd2(dt2, mk2(du0, du1), mk2(ur, umx)), nB = madd2(dt2, mk2(du2, du3), mk2(umy, umz));
            const F2 a2 = splat2(a);
            const F2 oA = madd2(a2, mk2(u00, u01), mul2(splat2(b), nA));
            const F2 oB = madd2(a2, mk2(u02, u03), mul2(splat2(b), nB));
            o0 = lo(oA); o1 = hi(oA); o2 = lo(oB); o3 = hi(oB);
        }
#else
        const float un0 = ur + dt * du0, un1 = umx + dt * du1, un2 = umy + dt * du2, un3 = umz + dt * du3;
        const float o0 = a * u00 + b * un0, o1 = a * u01 + b * un1, o2 = a * u02 + b * un2, o3 = a * u03 + b * un3;
#endif
        const float r = fmaxq(o0, floor_);
#if NB_ARITH_FAST
        // one reciprocal for the three velocities and the max speed; the speed cap compares the
        // squared speed and takes a root only for the capped cells
        const float ri = rcp_fast(r);
        float vx = o1 * ri, vy = o2 * ri, vz = o3 * ri;
        const float s2 = (vx * vx + vy * vy) + vz * vz;
        if (s2 > vmax * vmax) {
            const float f = vmax * rsqrtf(s2);
            vx = vx * f; vy = vy * f; vz = vz * f;
        }
#else
        float vx = o1 / r, vy = o2 / r, vz = o3 / r;
        const float sp = sqrtf((vx * vx + vy * vy) + vz * vz);
        if (sp > vmax) {
            const float f = vmax / sp;
            vx = vx * f; vy = vy * f; vz = vz * f;
        }
#endif
        const float m1 = r * vx, m2 = r * vy, m3 = r * vz;
        if (inside) {
            L.out[0][cell] = r;
            L.out[1][cell] = m1;
            L.out[2][cell] = m2;
            L.out[3][cell] = m3;
            if (STAGE2 && L.smax_bits) {         // nebula3d.py:158-162 on the new state
#if NB_ARITH_FAST
                const float v = fabsf(m1 * ri) + fabsf(m2 * ri) + fabsf(m3 * ri) + c[own].y;
#else
                const float v = fabsf(m1 / r) + fabsf(m2 / r) + fabsf(m3 / r) + c[own].y;
#endif
                vmax_local = fmaxq(v, vmax_local);
            }
        }
    }
    if (failed) return;
    if (STAGE2 && L.smax_bits) {                 // this tile's CFL max speed into its instance
        for (int o = 16; o > 0; o >>= 1) vmax_local = fmaxr(vmax_local, __shfl_xor_sync(0xffffffffu, vmax_local, o));
        float* red = reinterpret_cast<float*>(fy);
        __syncthreads();
        if (tk == 0) red[tj] = vmax_local;
        __syncthreads();
        if (tid == 0) {
            float m = 0.0f;
            for (int w = 0; w < TJ; ++w) m = fmaxr(m, red[w]);
            atomicMax(L.smax_bits, __float_as_uint(m));
        }
    }
}

// a TMA wait gave up: record it, let both slots' copies land (bounded waits), leave
template <int TJ>
__device__ __forceinline__ void hydro_abort(unsigned char* smem, unsigned* status, unsigned ph0, unsigned limit) {
    using SM = HydroSmem<TJ>;
    uint64_t* bar = reinterpret_cast<uint64_t*>(smem + SM::FIXED - SM::BAR_BYTES);
    if (threadIdx.x == 0) {                      // the one load that may still be in flight
        atomicOr(status, NB_DEV_TMA_TIMEOUT);
        mbar_wait_limited(&bar[0], ph0, &limit);
    }
    __syncthreads();
}

// the barriers, and the block's work rotation (hydro_tile) from the slot of its first warp: the
// blocks resident on an SM occupy different groups of 8 slots and so take different rotations
template <int TJ>
__device__ __forceinline__ void hydro_init_bars(unsigned char* smem, int* rot) {
    using SM = HydroSmem<TJ>;
    uint64_t* bar = reinterpret_cast<uint64_t*>(smem + SM::FIXED - SM::BAR_BYTES);
    if (threadIdx.x == 0) {
        mbar_init(&bar[0], 1);
        mbar_init(&bar[1], 1);
        fence_mbar_init();
        *rot = (int)((warp_slot() >> 3) & 3u);
    }
    __syncthreads();
}

template <int SOLVER, int LIM, int TJ, bool STAGE2, bool I32>
__global__ void __launch_bounds__(TK * TJ, NB_HYDRO_MINB) hydro_stage_kernel(const HydroLaunch L) {
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ int rot;
    hydro_init_bars<TJ>(smem, &rot);
    unsigned ph0 = 0;
    bool failed = false;
    hydro_tile<SOLVER, LIM, TJ, STAGE2, I32>(L, blockIdx.x, smem, ph0, failed, rot);
    if (failed) hydro_abort<TJ>(smem, L.status, ph0, L.wait_limit);
}

// Persistent batched stage: blocks take (instance, tile) work items from a list spanning many
// instances of different sizes, in list order, through one atomic counter (reset by the
// batched control kernel before every step).  A block whose bounded wait gave up computes nothing
// more: it keeps taking items and flags the instance of each one it leaves undone, so every
// instance with an unwritten tile reports NB_DEV_TMA_TIMEOUT.
#ifndef NB_HYDRO_BATCH_MINB
#define NB_HYDRO_BATCH_MINB 3            // records in global memory: their loaded fields need the 80-register budget
#endif
template <int SOLVER, int LIM, int TJ, bool STAGE2, bool I32>
__global__ void __launch_bounds__(TK * TJ, NB_HYDRO_BATCH_MINB)
hydro_batch_kernel(const HydroLaunch* __restrict__ Ls, const int2* __restrict__ work, int n_work,
                   unsigned* counter) {
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ int item, rot;
    hydro_init_bars<TJ>(smem, &rot);
    unsigned ph0 = 0;
    bool failed = false;                         // block-uniform (hydro_tile sets it after a barrier)
    const HydroLaunch* last = nullptr;
    for (;;) {
        if (threadIdx.x == 0) item = (int)atomicAdd(counter, 1u);
        __syncthreads();
        const int it = item;
        if (it >= n_work) break;
        const int2 w = work[it];
        if (!Ls[w.x].active) {                   // an idle slot of the batch: nothing to do
            __syncthreads();
            continue;
        }
        last = &Ls[w.x];
        hydro_tile<SOLVER, LIM, TJ, STAGE2, I32>(*last, w.y, smem, ph0, failed, rot);
        if (failed) break;
        __syncthreads();
    }
    if (failed && last) {
        hydro_abort<TJ>(smem, last->status, ph0, last->wait_limit);
        // the items this block would still have taken are left undone: flag their instances (the
        // counter grows by one per turn, so the loop ends)
        if (threadIdx.x == 0)
            for (unsigned it; (it = atomicAdd(counter, 1u)) < (unsigned)n_work;)
                atomicOr(Ls[work[it].x].status, NB_DEV_TMA_TIMEOUT);
    }
}

// The same persistent stage with the stage records in the kernel parameter (batches of at most
// NB_BATCH_PARAM_MAX instances, 32-bit offsets): a record's fields come from the constant bank,
// as the single-instance kernel's do, so it fits 64 registers and 4 blocks / SM.  The active flags
// (changed between graph replays) and the status words are read from the device copy Lg.
template <int SOLVER, int LIM, int TJ, bool STAGE2>
__global__ void __launch_bounds__(TK * TJ, NB_HYDRO_MINB)
hydro_batch_param_kernel(const __grid_constant__ NbBatchRecords R, const HydroLaunch* __restrict__ Lg,
                         const int2* __restrict__ work, int n_work, unsigned* counter) {
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ int item, rot;
    hydro_init_bars<TJ>(smem, &rot);
    unsigned ph0 = 0;
    bool failed = false;                         // block-uniform (hydro_tile sets it after a barrier)
    int last = -1;
    for (;;) {
        if (threadIdx.x == 0) item = (int)atomicAdd(counter, 1u);
        __syncthreads();
        const int it = item;
        if (it >= n_work) break;
        const int2 w = work[it];
        if (!Lg[w.x].active) {                   // an idle slot of the batch: nothing to do
            __syncthreads();
            continue;
        }
        last = w.x;
        hydro_tile<SOLVER, LIM, TJ, STAGE2, true>(R.L[w.x], w.y, smem, ph0, failed, rot);
        if (failed) break;
        __syncthreads();
    }
    if (failed && last >= 0) {
        hydro_abort<TJ>(smem, Lg[last].status, ph0, Lg[last].wait_limit);
        if (threadIdx.x == 0)                    // flag the instances of the items left undone
            for (unsigned it; (it = atomicAdd(counter, 1u)) < (unsigned)n_work;)
                atomicOr(Lg[work[it].x].status, NB_DEV_TMA_TIMEOUT);
    }
}

template <int SOLVER, int LIM, int TJ, bool STAGE2, bool I32>
cudaError_t run_kernel(const HydroLaunch& L, cudaStream_t s) {
    auto kern = hydro_stage_kernel<SOLVER, LIM, TJ, STAGE2, I32>;
    const int smem = HydroSmem<TJ>::bytes(L.nstars_host);
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e == cudaSuccess)                        // the largest shared-memory carveout: 4 blocks of ~57 KB per SM
        e = cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout, cudaSharedmemCarveoutMaxShared);
    if (e != cudaSuccess) return e;
    const int blocks = L.tiles_k * L.tiles_j * L.n_chunks;
    kern<<<blocks, TK * TJ, smem, s>>>(L);
    return cudaGetLastError();
}

template <int SOLVER, int LIM, int TJ>
cudaError_t run_stage(const HydroLaunch& L, cudaStream_t s) {
    const bool s2 = L.smax_bits || L.u0[0] != L.in[0];
    if (L.idx32) return s2 ? run_kernel<SOLVER, LIM, TJ, true, true>(L, s) : run_kernel<SOLVER, LIM, TJ, false, true>(L, s);
    return s2 ? run_kernel<SOLVER, LIM, TJ, true, false>(L, s) : run_kernel<SOLVER, LIM, TJ, false, false>(L, s);
}

template <int SOLVER, int LIM, int TJ, bool STAGE2, bool I32>
cudaError_t run_batch_kernel(const HydroLaunch* Ls, const NbBatchRecords* rec, const int2* work, int n_work,
                             unsigned* counter, int max_stars, int grid, cudaStream_t s) {
    const int smem = HydroSmem<TJ>::bytes(max_stars);
    if (I32 && rec) {
        auto kern = hydro_batch_param_kernel<SOLVER, LIM, TJ, STAGE2>;
        cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout,
                                     cudaSharedmemCarveoutMaxShared);
        if (e != cudaSuccess) return e;
        kern<<<grid, TK * TJ, smem, s>>>(*rec, Ls, work, n_work, counter);
        return cudaGetLastError();
    }
    auto kern = hydro_batch_kernel<SOLVER, LIM, TJ, STAGE2, I32>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout, cudaSharedmemCarveoutMaxShared);
    if (e != cudaSuccess) return e;
    kern<<<grid, TK * TJ, smem, s>>>(Ls, work, n_work, counter);
    return cudaGetLastError();
}

template <int SOLVER, int LIM, int TJ>
cudaError_t run_batch(const HydroLaunch* Ls, const NbBatchRecords* rec, const int2* work, int n_work,
                      unsigned* counter, int max_stars, int stage2, int idx32, int grid, cudaStream_t s) {
    if (idx32)
        return stage2 ? run_batch_kernel<SOLVER, LIM, TJ, true, true>(Ls, rec, work, n_work, counter, max_stars, grid, s)
                      : run_batch_kernel<SOLVER, LIM, TJ, false, true>(Ls, rec, work, n_work, counter, max_stars, grid, s);
    return stage2 ? run_batch_kernel<SOLVER, LIM, TJ, true, false>(Ls, nullptr, work, n_work, counter, max_stars, grid, s)
                  : run_batch_kernel<SOLVER, LIM, TJ, false, false>(Ls, nullptr, work, n_work, counter, max_stars, grid, s);
}

}  // namespace

int nb_hydro_tile_j() { return NB_HYDRO_TJ; }

// resident blocks per SM of the persistent stage kernel (sizes its grid)
int nb_hydro_batch_blocks_per_sm(int solver, int limiter, int max_stars, int idx32, int params) {
    constexpr int TJ = NB_HYDRO_TJ;
    const int smem = HydroSmem<TJ>::bytes(max_stars);
    auto occ = [&](auto kern) {
        int n = 0;
        if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem) != cudaSuccess ||
            cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout, cudaSharedmemCarveoutMaxShared) !=
                cudaSuccess ||
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, kern, TK * TJ, smem) != cudaSuccess) {
            cudaGetLastError();
            return 0;
        }
        return n;
    };
    int n;
    if (idx32 && params) {
        if (solver == NB_SOLVER_RUSANOV)
            n = occ(hydro_batch_param_kernel<NB_SOLVER_RUSANOV, 0, TJ, true>);
        else if (limiter == NB_LIM_VANLEER)
            n = occ(hydro_batch_param_kernel<NB_SOLVER_HLL, NB_LIM_VANLEER, TJ, true>);
        else if (limiter == NB_LIM_MC)
            n = occ(hydro_batch_param_kernel<NB_SOLVER_HLL, NB_LIM_MC, TJ, true>);
        else
            n = occ(hydro_batch_param_kernel<NB_SOLVER_HLL, NB_LIM_MINMOD, TJ, true>);
        return n > 0 ? n : NB_HYDRO_MINB;
    }
    if (solver == NB_SOLVER_RUSANOV)
        n = idx32 ? occ(hydro_batch_kernel<NB_SOLVER_RUSANOV, 0, TJ, true, true>)
                  : occ(hydro_batch_kernel<NB_SOLVER_RUSANOV, 0, TJ, true, false>);
    else if (limiter == NB_LIM_VANLEER)
        n = idx32 ? occ(hydro_batch_kernel<NB_SOLVER_HLL, NB_LIM_VANLEER, TJ, true, true>)
                  : occ(hydro_batch_kernel<NB_SOLVER_HLL, NB_LIM_VANLEER, TJ, true, false>);
    else if (limiter == NB_LIM_MC)
        n = idx32 ? occ(hydro_batch_kernel<NB_SOLVER_HLL, NB_LIM_MC, TJ, true, true>)
                  : occ(hydro_batch_kernel<NB_SOLVER_HLL, NB_LIM_MC, TJ, true, false>);
    else
        n = idx32 ? occ(hydro_batch_kernel<NB_SOLVER_HLL, NB_LIM_MINMOD, TJ, true, true>)
                  : occ(hydro_batch_kernel<NB_SOLVER_HLL, NB_LIM_MINMOD, TJ, true, false>);
    return n > 0 ? n : NB_HYDRO_BATCH_MINB;
}

cudaError_t nb_launch_hydro(const HydroLaunch& L, int solver, int limiter, cudaStream_t s) {
    constexpr int TJ = NB_HYDRO_TJ;
    if (solver == NB_SOLVER_RUSANOV) return run_stage<NB_SOLVER_RUSANOV, 0, TJ>(L, s);
    switch (limiter) {
        case NB_LIM_VANLEER: return run_stage<NB_SOLVER_HLL, NB_LIM_VANLEER, TJ>(L, s);
        case NB_LIM_MC: return run_stage<NB_SOLVER_HLL, NB_LIM_MC, TJ>(L, s);
        default: return run_stage<NB_SOLVER_HLL, NB_LIM_MINMOD, TJ>(L, s);
    }
}

cudaError_t nb_launch_hydro_batch(const HydroLaunch* Ls, const NbBatchRecords* rec, const int2* work, int n_work,
                                  unsigned* counter, int max_stars, int stage2, int idx32, int solver, int limiter,
                                  int grid, cudaStream_t s) {
    constexpr int TJ = NB_HYDRO_TJ;
    if (solver == NB_SOLVER_RUSANOV)
        return run_batch<NB_SOLVER_RUSANOV, 0, TJ>(Ls, rec, work, n_work, counter, max_stars, stage2, idx32, grid, s);
    switch (limiter) {
        case NB_LIM_VANLEER:
            return run_batch<NB_SOLVER_HLL, NB_LIM_VANLEER, TJ>(Ls, rec, work, n_work, counter, max_stars, stage2, idx32,
                                                                grid, s);
        case NB_LIM_MC:
            return run_batch<NB_SOLVER_HLL, NB_LIM_MC, TJ>(Ls, rec, work, n_work, counter, max_stars, stage2, idx32, grid,
                                                           s);
        default:
            return run_batch<NB_SOLVER_HLL, NB_LIM_MINMOD, TJ>(Ls, rec, work, n_work, counter, max_stars, stage2, idx32,
                                                               grid, s);
    }
}
