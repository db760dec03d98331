// Point operators of the reconstruction shared by the fused passes and the
// reference-compatible single-stage kernels.
#pragma once
#include "ctdm_common.cuh"
#include "kernels.cuh"

namespace ctdm {

// calculate_n3D (cTDM/Recon_kernel.cu:305-342): n = n_med sqrt(1 + F/(-k^2)), the
// principal root, then Re n >= n_med and Im n >= 0.  The root is evaluated in the
// cancellation-free form (the larger of a, |b| from the half-sum formula, the
// other from d / 2x); it is the same function as the reference's expression.
__device__ __forceinline__ float2 est_n(float2 F, float k2, float nm)
{
    const float c = F.x / (-k2) + 1.0f, d = F.y / (-k2);
    const float mod = hypotf(c, d);
    float a, b;
    if (d == 0.0f) {
        a = sqrtf(fmaxf(c, 0.0f));
        b = 0.0f;
    } else if (c >= 0.0f) {
        a = sqrtf((mod + c) * 0.5f);
        b = d / (2.0f * a);
    } else {
        b = sqrtf((mod - c) * 0.5f);
        a = fabsf(d) / (2.0f * b);
        if (d < 0.0f) b = -b;
    }
    float nr = a * nm, ni = b * nm;
    if (nr < nm) nr = nm;
    if (ni < 0.0f) ni = 0.0f;
    return make_float2(nr, ni);
}

// The same root for an unscaled inverse-transform value v: c = 1 + v s1 with
// s1 = -1/(R^3 k^2) folding the 1/R^3 normalisation and the division by -k^2.
// Evaluated without division or branch: with h = (|z| + |c|) / 2, the parts of
// the principal root are sqrt(h) and |d| / (2 sqrt(h)); the first is the real
// part when c >= 0 and the imaginary part (sign of d) when c < 0.  Square roots
// come from the hardware reciprocal square root (sqrt(h) = h rsqrt(h)); a few ulp
// against the correctly rounded form, far inside the loop's float32 error.
__device__ __forceinline__ float2 est_n_scaled(float2 v, float s1, float nm)
{
    const float c = fmaf(v.x, s1, 1.0f), d = v.y * s1;
    const float m2 = fmaf(c, c, d * d);
    const float mod = m2 > 0.0f ? m2 * rsqrtf(m2) : 0.0f;
    const float h = 0.5f * (mod + fabsf(c));
    const float rh = h > 0.0f ? rsqrtf(h) : 0.0f;
    const float big = h * rh, small = 0.5f * fabsf(d) * rh;
    const bool pos = c >= 0.0f;
    const float a = pos ? big : small;
    const float bm = pos ? small : (d == 0.0f ? 0.0f : big);
    const float b = copysignf(bm, d);
    return make_float2(fmaxf(a * nm, nm), fmaxf(b * nm, 0.0f));
}

// Modify_F3D with the constants folded: f = ((nr^2 - ni^2) s2 + k^2, 2 nr ni s2),
// s2 = -k^2 / n_med^2.
__device__ __forceinline__ float2 modify_f_scaled(float2 n, float s2, float k2)
{
    return make_float2(fmaf(n.x * n.x - n.y * n.y, s2, k2), 2.0f * n.x * n.y * s2);
}

// Brings the line containing p towards L2 without holding a register for the data
// (the accelerated loop's previous iterate, read after the transforms that follow).
__device__ __forceinline__ void prefetch_l2(const void *p)
{
    asm volatile("prefetch.global.L2 [%0];" ::"l"(p));
}

// Nesterov momentum on the projected iterate: w = x + beta (x - x_prev).
__device__ __forceinline__ float2 momentum_step(float2 x, float2 prev, float beta)
{
    return make_float2(fmaf(beta, x.x - prev.x, x.x), fmaf(beta, x.y - prev.y, x.y));
}

// Modify_F3D (cTDM/Recon_kernel.cu:370-383), called with n_med^2.
__device__ __forceinline__ float2 modify_f(float2 n, float k2, float nm2)
{
    return make_float2(((n.x * n.x - n.y * n.y) / nm2 - 1.0f) * (-k2), (n.x * n.y * 2.0f) / nm2 * (-k2));
}

// Voxel z index of fillEdwardSphere (cTDM/Recon_kernel.cu:187-229, cuRound :236):
// nz = mod(round_half_away((f_z - f_z0)/df), R) with
// f_z = sqrt(fm0^2 - (fx^2 + fy^2)), fx = ii df + fx0, fy = jj df + fy0; no sample
// where the radicand is negative.  The rule is defined in IEEE double without
// contraction.  A float evaluation in units of df decides it whenever its result is
// farther from a decision boundary than twice a bound on its error; otherwise the
// double rule runs.  The bound (u = 2^-24, F = fm0/df, the float constants rounded
// from double): the radicand's error is at most E = 10 u F^2 (the constants' rounding,
// fx0/df and fy0/df carried through the squares, the squares, the sum and the
// difference, each within u of its value, every term at most F^2), so
// |sqrt(rads) - sqrt(RAD)| <= E / fzs + u fzs, and with the rounding of fz0/df, of
// t = fzs - fz0s and of its fraction the index fraction is within
// u (E / (u fzs) + fzs + |fz0s| + |t| + 1) of the double rule's.  For 256^3 at
// 0.1 um voxels (F = 64.3) that is about 1e-4 at the cap's centre instead of a fixed
// 0.02 margin: the double rule runs for well under 1% of the samples instead of 4%,
// whose divergent FP64 division and square root dominated the mapping.
// ewald_nz_signed returns the unwrapped index (kNoSample where the radicand is
// negative) and fz (1/m) for the value; ewald_nz wraps it into [0, R).
constexpr int kNoSample = -0x40000000;
__device__ __forceinline__ int ewald_nz_signed(int ii, int jj, const AngleGeom &g, double df, double fm02,
                                               float fm02s, float &fz)
{
    const float fxs = (float)ii + g.fx0s, fys = (float)jj + g.fy0s;
    const float rads = fm02s - (fxs * fxs + fys * fys);
    const float er = 5.9604645e-7f * fm02s;   // E = 10 u F^2
    if (rads < -1.0f - er) return kNoSample;
    if (rads >= fmaxf(1.0f, er)) {
        const float fzs = sqrtf(rads);
        const float t = fzs - g.fz0s;
        const float fl = floorf(t);
        const float fr = t - fl;
        const float bound = 1.1920929e-7f * (er * 16777216.0f / fzs + fzs + fabsf(g.fz0s) + fabsf(t) + 1.0f);
        if (fabsf(fr - 0.5f) > bound) {
            fz = fzs * (float)df;
            return (fr > 0.5f) ? (int)fl + 1 : (int)fl;
        }
    }
    const double fx = __dadd_rn(__dmul_rn((double)ii, df), g.fx0);
    const double fy = __dadd_rn(__dmul_rn((double)jj, df), g.fy0);
    const double s = __dadd_rn(__dmul_rn(fx, fx), __dmul_rn(fy, fy));
    const double rad = __dsub_rn(fm02, s);
    if (rad < 0.0) return kNoSample;
    const double fzd = __dsqrt_rn(rad);
    const double t = __ddiv_rn(__dsub_rn(fzd, g.fz0), df);
    const double rn = t > 0.0 ? floor(__dadd_rn(t, 0.5)) : ceil(__dsub_rn(t, 0.5));
    fz = (float)fzd;
    return (int)rn;
}

__device__ __forceinline__ int ewald_nz(int ii, int jj, const AngleGeom &g, double df, double fm02, float fm02s,
                                        int R, float &fz)
{
    const int nz = ewald_nz_signed(ii, jj, g, df, fm02, fm02s, fz);
    return nz == kNoSample ? -1 : imod(nz, R);
}

}  // namespace ctdm
