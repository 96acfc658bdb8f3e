// Pair arithmetic shared by the single-system and batched kernels.
//
// * ref64_*: the reference's FP64 arithmetic, operation for operation, with explicit
//   round-to-nearest intrinsics so the compiler cannot contract a multiply-add into an FMA
//   (the reference is built in ISO C++ mode without contraction).  A pair evaluated here gives
//   bitwise the value FField_MDBAS computes for it (FField_MDBAS.cpp:366-414, Tools.hpp:151-224,
//   PerConditions.cpp:244-285).
// * mixed_*: FP32 pair terms on an exact minimum-image displacement taken from 32-bit
//   fixed-point coordinates (coordinate / box * 2^32): unsigned subtraction wraps modulo the box,
//   which is the minimum image, and the integer difference is exact.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "dev_types.hpp"

namespace mcg {

// Tools::rint (Tools.hpp:221-224): half away from zero through an int cast.
__device__ __forceinline__ double ref64_rint(double x) {
    double t = (x >= 0.0) ? __dadd_rn(x, 0.5) : __dsub_rn(x, 0.5);
    return (double)__double2int_rz(t);
}

// d -= L * rint(rL * d)
__device__ __forceinline__ double ref64_mic(double d, double L, double rL) {
    return __dsub_rn(d, __dmul_rn(L, ref64_rint(__dmul_rn(rL, d))));
}

// Tools::distance2(a1, a2): delta = a2 - a1, MIC, r^2 = (dx^2 + dy^2) + dz^2.
__device__ __forceinline__ double ref64_dist2(double ax, double ay, double az, double bx, double by, double bz,
                                              const PbcDev& p, double* d = nullptr) {
    double dx = __dsub_rn(bx, ax), dy = __dsub_rn(by, ay), dz = __dsub_rn(bz, az);
    if (p.type != 0) {
        dx = ref64_mic(dx, p.L[0], p.rL[0]);
        dy = ref64_mic(dy, p.L[1], p.rL[1]);
        dz = ref64_mic(dz, p.L[2], p.rL[2]);
    }
    if (d) { d[0] = dx; d[1] = dy; d[2] = dz; }
    return __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz));
}

// computeEelec / computeEvdw and the switch of computeNonBonded_switch, unscaled:
// el = qi qj / r * S, vd = eps_i eps_j (x^12 - x^6) * S with x = (sig_i + sig_j) / r.
__device__ __forceinline__ void ref64_pair(double r2, double qi, double qj, double ei, double ej, double si,
                                           double sj, bool do_switch, const CutDev& c, double& el, double& vd) {
    double r = __dsqrt_rn(r2);
    double rt = __ddiv_rn(1.0, r);
    double pe = __dmul_rn(__dmul_rn(qi, qj), rt);
    double x = __dmul_rn(__dadd_rn(si, sj), rt);
    double x12 = x;
#pragma unroll
    for (int k = 0; k < 11; k++) x12 = __dmul_rn(x12, x);
    double x6 = x;
#pragma unroll
    for (int k = 0; k < 5; k++) x6 = __dmul_rn(x6, x);
    double pv = __dmul_rn(__dmul_rn(ei, ej), __dsub_rn(x12, x6));
    if (do_switch && r2 > c.n2) {
        double s1 = __dsub_rn(c.c2, r2);
        double f = __dmul_rn(__dmul_rn(__dmul_rn(s1, s1), __dsub_rn(__dadd_rn(c.c2, __dmul_rn(2.0, r2)),
                                                                      __dmul_rn(3.0, c.n2))), c.sw2);
        pe = __dmul_rn(pe, f);
        pv = __dmul_rn(pv, f);
    }
    el = pe;
    vd = pv;
}

// ---- fixed-point coordinates --------------------------------------------------------------
// u = wrapped(x) / L in [-1/2, 1/2) scaled by 2^32 and stored modulo 2^32.
__device__ __forceinline__ uint32_t to_fixed(double x, double rL) {
    double u = x * rL;
    u -= rint(u);                               // [-0.5, 0.5]
    long long v = __double2ll_rn(u * 4294967296.0);
    return (uint32_t)(unsigned long long)v;
}

// exact minimum-image displacement b - a in box units of 2^-32, converted to Angstrom (FP32).
// The scale L/2^32 is a float-float pair (Lh + Ll): a scale rounded to float would shrink or
// stretch every distance by the same factor, a systematic error that the virial of an unrelaxed
// configuration amplifies about fifty-fold in the total energy.
__device__ __forceinline__ float fixed_delta(uint32_t a, uint32_t b, float Lh, float Ll) {
    const float f = __int2float_rn((int)(b - a));
    return fmaf(f, Lh, f * Ll);
}

// FP32 switched LJ + Coulomb on r^2 (unscaled el, vd as in ref64_pair).  The charge product is
// a float-float pair (qq + qq_lo): per-type products rounded to float are systematic biases that
// the cancellation between positive and negative Coulomb terms would amplify to ~1e-6 of the
// total.  ee = eps_i eps_j, ss = (sig_i + sig_j)^2.
__device__ __forceinline__ void mixed_pair(float r2, float qq, float qq_lo, float ee, float ss, bool do_switch,
                                           const CutDev& c, float& el, float& vd, float ee_lo = 0.f, float ss_lo = 0.f) {
    float rinv = rsqrtf(r2);
    rinv = rinv * fmaf(-0.5f * r2 * rinv, rinv, 1.5f);   // one Newton step on the hardware estimate
    const float ri2 = rinv * rinv;
    float x2 = fmaf(ss, ri2, ss_lo * ri2);               // (sig_i+sig_j)^2 / r^2, float-float constant
    float x6 = x2 * x2 * x2;
    float f = 1.0f;
    if (do_switch && r2 > c.n2f) {
        float s1 = c.c2f - r2;
        f = s1 * s1 * (c.c2f + 2.0f * r2 - 3.0f * c.n2f) * c.sw2f;
    }
    el = fmaf(qq, rinv, qq_lo * rinv) * f;
    const float l = x6 * x6 - x6;
    vd = fmaf(ee, l, ee_lo * l) * f;
}

// float-float product of two float-float values (hi parts exact by FMA, cross terms rounded)
__device__ __forceinline__ void ff_mul(float ah, float al, float bh, float bl, float& ph, float& pl) {
    ph = ah * bh;
    pl = fmaf(ah, bh, -ph) + fmaf(ah, bl, al * bh);
}

// TwoSum: s + e == a + b exactly
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
    s = a + b;
    float bp = s - a;
    e = (a - (s - bp)) + (b - bp);
}

// Error-free FP32 accumulation (Kahan-Babuska / Neumaier): sum + comp carries ~48 bits.
struct F32Acc {
    float s = 0.f, c = 0.f;
    __device__ __forceinline__ void add(float v) {
        float t = s + v;
        c += (fabsf(s) >= fabsf(v)) ? ((s - t) + v) : ((v - t) + s);
        s = t;
    }
    __device__ __forceinline__ double value() const { return (double)s + (double)c; }
};

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

}  // namespace mcg

namespace mcg {

// Energy change of one pair when one side moves by m (d_new = d_old - m), FP32, in iu.
// qk = 332.0716*418.4*qi*qj, e4 = 4*eps_i*eps_j, ss = (sig_i+sig_j)^2.
// Coulomb (the large term) is differenced analytically so its error is relative to the change,
// not to the pair energy: with u = r^2 and du = u_new - u_old = -m.(d_old + d_new),
//   1/r_new - 1/r_old = -du (rn ro)^2 / (rn + ro)        (rn, ro = rsqrt(u_new), rsqrt(u_old))
//   S_b - S_a = sw2 du' [2 A_a^2 - (A_a + A_b) B_b],  A = c2 - u, B = c2 + 2u - 3 n2
// on the switch polynomial (u clamped to [n2, c2]).  LJ is small at these distances and is
// differenced directly.  Pairs crossing the cutoff fall back to the direct difference.
// npair counts pair interactions (inside the cutoff before or after the move).  Straight-line
// code: a pair outside the cutoff before and after gets switch factors 0 and contributes +-0, so
// a warp whose lanes hold pairs in different regions (inner, switch, outside, crossing the cutoff)
// executes one path, and independent calls interleave.  Needs r > 0 (distinct atoms).
__device__ __forceinline__ float mixed_pair_delta(float dox, float doy, float doz, float mx, float my, float mz,
                                                  float qk, float e4, float ss, const CutDev& c, int& npair) {
    const float dnx = dox - mx, dny = doy - my, dnz = doz - mz;
    const float uo = fmaf(dox, dox, fmaf(doy, doy, doz * doz));
    const float un = fmaf(dnx, dnx, fmaf(dny, dny, dnz * dnz));
    const bool io = uo <= c.c2f, in = un <= c.c2f;
    npair += (io || in) ? 1 : 0;
    const float ro = rsqrtf(uo), rn = rsqrtf(un);
    // switch S(u) = (c2-u)^2 (c2+2u-3n2) sw2 above n2, 1 below; evaluated on u clamped to [n2, c2]
    const float ua = fmaxf(uo, c.n2f), ub = fmaxf(un, c.n2f);
    const float Aa = c.c2f - ua, Ab = c.c2f - ub;
    const float k3 = c.c2f - 3.0f * c.n2f;
    const float Ba = fmaf(2.0f, ua, k3), Bb = fmaf(2.0f, ub, k3);
    const float so = io ? (uo <= c.n2f ? 1.0f : Aa * Aa * Ba * c.sw2f) : 0.0f;
    const float sn = in ? (un <= c.n2f ? 1.0f : Ab * Ab * Bb * c.sw2f) : 0.0f;
    // Lennard-Jones, differenced directly (small at these distances)
    const float xo = ss * (ro * ro), xn = ss * (rn * rn);
    const float xo3 = xo * xo * xo, xn3 = xn * xn * xn;
    const float d_lj = fmaf(e4 * fmaf(xn3, xn3, -xn3), sn, -(e4 * fmaf(xo3, xo3, -xo3) * so));
    // Coulomb: analytic difference when both ends are inside the cutoff
    //   1/r_new - 1/r_old = -du (rn ro)^2 / (rn + ro),  du = u_new - u_old = -m.(d_old + d_new)
    //   S_b - S_a = sw2 du' [2 A_a^2 - (A_a + A_b) B_b] on the clamped u (du' = du when both are above n2)
    const float du = -fmaf(mx, dox + dnx, fmaf(my, doy + dny, mz * (doz + dnz)));
    const float p = ro * rn;
    const float dinv = __fdividef(-du * p * p, ro + rn);
    const float dd = (uo > c.n2f && un > c.n2f) ? du : (ub - ua);
    const float ds = c.sw2f * dd * fmaf(2.0f * Aa, Aa, -(Aa + Ab) * Bb);
    const float c_both = qk * fmaf(dinv, sn, ro * ds);
    const float c_one = qk * fmaf(rn, sn, -ro * so);
    return d_lj + ((io && in) ? c_both : c_one);
}

// mixed_pair_delta for the batched sweep, with u clamped to [n2, c2] in the switch polynomial.
// The switch is used unnormalised, P(u) = A^2 B (A = c2 - u, B = 2u + c2 - 3 n2), and the caller
// passes qk and e4 already multiplied by sw2 = 1 / (c2 - n2)^3, so S = P sw2 without a multiply per
// pair.  P is then (c2 - n2)^3 below n2 (S = 1 to a relative 6e-8) and exactly 0 beyond rc, so no
// select is needed.  The analytic differences
//   1/r_n - 1/r_o = -du (r_o r_n)^2 / (r_o + r_n)
//   P_n - P_o = du' [2 A_o^2 - (A_o + A_n) B_n]   (du' = u_n - u_o on the clamped values)
// are exact algebra for any clamped pair, so one formula covers pairs inside, crossing and beyond
// the cutoff (beyond: P_o = P_n = 0 and the pair contributes 0).  du' is the accurate
// -m.(d_o + d_n) when both ends lie inside the switch region (ends on its boundaries included, where
// the two agree), the clamped difference otherwise.
__device__ __forceinline__ float mixed_pair_delta_clamped(float dox, float doy, float doz, float mx, float my, float mz,
                                                          float qk_sw, float e4_sw, float ss, float c2, float n2, float k3,
                                                          int& npair) {
    // The old and new ends of the pair are the two halves of float2 values, so the work both ends
    // share takes one sm_100+ packed instruction; every operation rounds as the scalar form would
    // (-x^3 is formed from -x, so x^6 - x^3 is the same single FMA).
    const float2 dx = make_float2(dox, dox - mx), dy = make_float2(doy, doy - my), dz = make_float2(doz, doz - mz);
    const float2 u = __ffma2_rn(dx, dx, __ffma2_rn(dy, dy, __fmul2_rn(dz, dz)));
    npair += fminf(u.x, u.y) <= c2 ? 1 : 0;
    const float2 r = make_float2(rsqrtf(u.x), rsqrtf(u.y));
    const float2 uc = make_float2(fminf(fmaxf(u.x, n2), c2), fminf(fmaxf(u.y, n2), c2));
    const float2 A = __ffma2_rn(uc, make_float2(-1.0f, -1.0f), make_float2(c2, c2));
    const float2 B = __ffma2_rn(make_float2(2.0f, 2.0f), uc, make_float2(k3, k3));
    const float2 P = __fmul2_rn(__fmul2_rn(A, A), B);
    // Lennard-Jones, differenced directly (small at these distances)
    const float2 nx = __fmul2_rn(make_float2(-ss, -ss), __fmul2_rn(r, r));
    const float2 nx3 = __fmul2_rn(__fmul2_rn(nx, nx), nx);
    const float2 w = __ffma2_rn(nx3, nx3, nx3);                   // x^6 - x^3 at both ends
    const float d_lj = e4_sw * fmaf(w.y, P.y, -(w.x * P.x));
    // Coulomb: qk (P_n / r_n - P_o / r_o) = qk ((1/r_n - 1/r_o) P_n + (P_n - P_o) / r_o)
    const float du = -fmaf(mx, dox + dx.y, fmaf(my, doy + dy.y, mz * (doz + dz.y)));
    const float p = r.x * r.y;
    const float dinv = __fdividef(-du * p * p, r.x + r.y);
    // both ends inside [ron^2, rc^2] exactly when the clamp left them unchanged
    const float dd = (uc.x == u.x && uc.y == u.y) ? du : (uc.y - uc.x);
    const float dp = dd * fmaf(2.0f * A.x, A.x, -(A.x + A.y) * B.y);
    return fmaf(qk_sw, fmaf(dinv, P.y, r.x * dp), d_lj);
}

// The same arithmetic without packed instructions: fewer live registers, for a kernel held to 64.
__device__ __forceinline__ float mixed_pair_delta_clamped_scalar(float dox, float doy, float doz, float mx, float my, float mz,
                                                          float qk_sw, float e4_sw, float ss, float c2, float n2, float k3,
                                                          int& npair) {
    const float dnx = dox - mx, dny = doy - my, dnz = doz - mz;
    const float uo = fmaf(dox, dox, fmaf(doy, doy, doz * doz));
    const float un = fmaf(dnx, dnx, fmaf(dny, dny, dnz * dnz));
    npair += fminf(uo, un) <= c2 ? 1 : 0;
    const float ro = rsqrtf(uo), rn = rsqrtf(un);
    const float ua = fminf(fmaxf(uo, n2), c2), ub = fminf(fmaxf(un, n2), c2);
    const float Aa = c2 - ua, Ab = c2 - ub;
    const float Ba = fmaf(2.0f, ua, k3), Bb = fmaf(2.0f, ub, k3);
    const float po = Aa * Aa * Ba, pn = Ab * Ab * Bb;
    // Lennard-Jones, differenced directly (small at these distances)
    const float xo = ss * (ro * ro), xn = ss * (rn * rn);
    const float xo3 = xo * xo * xo, xn3 = xn * xn * xn;
    const float d_lj = e4_sw * fmaf(fmaf(xn3, xn3, -xn3), pn, -(fmaf(xo3, xo3, -xo3) * po));
    // Coulomb: qk (P_n / r_n - P_o / r_o) = qk ((1/r_n - 1/r_o) P_n + (P_n - P_o) / r_o)
    const float du = -fmaf(mx, dox + dnx, fmaf(my, doy + dny, mz * (doz + dnz)));
    const float p = ro * rn;
    const float dinv = __fdividef(-du * p * p, ro + rn);
    // both ends inside [ron^2, rc^2] exactly when the clamp left them unchanged
    const float dd = (ua == uo && ub == un) ? du : (ub - ua);
    const float dp = dd * fmaf(2.0f * Aa, Aa, -(Aa + Ab) * Bb);
    return fmaf(qk_sw, fmaf(dinv, pn, ro * dp), d_lj);
}

// the packed or the scalar form (the same values)
template <bool PACKED>
__device__ __forceinline__ float pair_delta(float dox, float doy, float doz, float mx, float my, float mz, float qk_sw,
                                            float e4_sw, float ss, float c2, float n2, float k3, int& npair) {
    if (PACKED) return mixed_pair_delta_clamped(dox, doy, doz, mx, my, mz, qk_sw, e4_sw, ss, c2, n2, k3, npair);
    return mixed_pair_delta_clamped_scalar(dox, doy, doz, mx, my, mz, qk_sw, e4_sw, ss, c2, n2, k3, npair);
}

// Block sums of two doubles (every thread passes its values; thread 0 of warp 0 writes out[0..1]).
__device__ __forceinline__ void block_reduce2(double a, double b, double* out) {
    __shared__ double sa[32], sb[32];
    a = warp_sum(a); b = warp_sum(b);
    int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    if (l == 0) { sa[w] = a; sb[w] = b; }
    __syncthreads();
    if (w == 0) {
        int nw = blockDim.x >> 5;
        a = l < nw ? sa[l] : 0.0; b = l < nw ? sb[l] : 0.0;
        a = warp_sum(a); b = warp_sum(b);
        if (l == 0) { out[0] = a; out[1] = b; }
    }
    __syncthreads();
}

// A lane's share of row i of the factored pair sums: q_i (ch + cl) and eps_i vs, into the lane's float-float totals
__device__ __forceinline__ void mix_row_flush(float4 pi, float ch, float cl, float vs, float& EH, float& EL, float& VH,
                                              float& VL) {
    float ph, pl, sm, er;
    ff_mul(pi.x, pi.y, ch, cl, ph, pl);
    two_sum(EH, ph, sm, er);
    EH = sm;
    EL += er + pl;
    two_sum(VH, pi.z * vs, sm, er);
    VH = sm;
    VL += er;
}

}  // namespace mcg
