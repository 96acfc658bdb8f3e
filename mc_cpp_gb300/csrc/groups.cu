// Group-pair form of the pruned Verlet rows and its energy kernel (see groups.hpp).
#include <algorithm>
#include <climits>
#include <string>
#include <type_traits>
#include <vector>

#include <cuda_runtime.h>

#include "engine.hpp"
#include "groups.hpp"
#include "pair_math.cuh"

namespace mcg {

#define GK(call)                                                                              \
    do {                                                                                      \
        cudaError_t e_ = (call);                                                              \
        if (e_ != cudaSuccess) return fail(MCG_ECUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

constexpr int GB_WARPS = 4;            // warps per CTA of the row build
constexpr int GH_BITS = 10;
constexpr int GH_SLOTS = 1 << GH_BITS; // hash slots per warp
constexpr int GH_MAX = GH_SLOTS / 2;   // partner groups per row, at most (keeps the probes short)
constexpr int GE_THREADS = 256;        // threads per CTA of the energy kernel

// Group rows from the per-atom rows, a warp per group.  The partner groups of the group's atoms
// are gathered into a per-warp hash table in shared memory (key: partner group, value: the mask
// of atom pairs), then compacted and sorted by partner group, so a row's entries and their order
// depend on the source rows' contents only.  A row with more than GH_MAX partner groups, or more
// than gcap, sets the overflow flag and is left empty (the host then disables the path).
__global__ void __launch_bounds__(GB_WARPS * 32) k_group_rows(const int* __restrict__ gstart, const int* __restrict__ gof,
                                                              int ngroup, const int* __restrict__ rows,
                                                              const int* __restrict__ lens, int cap, int2* __restrict__ grow,
                                                              int* __restrict__ glen, int gcap,
                                                              unsigned long long* __restrict__ misc) {
    __shared__ int s_key[GB_WARPS][GH_SLOTS];
    __shared__ int s_msk[GB_WARPS][GH_SLOTS];
    __shared__ int s_cnt[GB_WARPS];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    int* key = s_key[w];
    int* msk = s_msk[w];
    for (int t = lane; t < GH_SLOTS; t += 32) { key[t] = -1; msk[t] = 0; }
    unsigned long long ent = 0, bits = 0;
    bool over = false;
    for (int g = blockIdx.x * GB_WARPS + w; g < ngroup; g += gridDim.x * GB_WARPS) {
        const int a0 = gstart[g], ni = gstart[g + 1] - a0;
        if (lane == 0) s_cnt[w] = 0;
        __syncwarp();
        for (int a = 0; a < ni; a++) {
            const int i = a0 + a, m = lens[i];
            const int* row = rows + (size_t)i * cap;
            for (int k = lane; k < m; k += 32) {
                const int j = row[k];
                const int h = gof[j];
                const int bit = 1 << (a * 4 + (j - gstart[h]));
                unsigned s = ((unsigned)h * 2654435761u) >> (32 - GH_BITS);
                for (int p = 0; p < GH_SLOTS; p++) {     // linear probing, bounded
                    const int old = atomicCAS(&key[s], -1, h);
                    if (old == -1 || old == h) {
                        if (old == -1) atomicAdd(&s_cnt[w], 1);
                        atomicOr(&msk[s], bit);
                        break;
                    }
                    s = (s + 1) & (GH_SLOTS - 1);
                }
            }
        }
        __syncwarp();
        const int cnt = s_cnt[w];
        if (cnt > GH_MAX || cnt > gcap) {
            over = true;
            if (lane == 0) glen[g] = 0;
        } else {
            // compact the occupied slots to the front (in place: a chunk is read before it is written,
            // and the write position never passes the read position)
            int out = 0;
            for (int base = 0; base < GH_SLOTS; base += 32) {
                const int kk = key[base + lane], mm = msk[base + lane];
                const unsigned occ = __ballot_sync(0xffffffffu, kk >= 0);
                __syncwarp();
                if (kk >= 0) {
                    const int p = out + __popc(occ & ((1u << lane) - 1u));
                    key[p] = kk;
                    msk[p] = mm;
                }
                out += __popc(occ);
                __syncwarp();
            }
            int P = 1;
            while (P < cnt) P <<= 1;
            for (int t = cnt + lane; t < P; t += 32) key[t] = INT_MAX;
            __syncwarp();
            // bitonic sort of (key, mask) by key over P entries
            for (int k = 2; k <= P; k <<= 1)
                for (int j = k >> 1; j > 0; j >>= 1) {
                    for (int t = lane; t < (P >> 1); t += 32) {
                        const int lo = ((t & ~(j - 1)) << 1) | (t & (j - 1)), hi = lo + j;
                        const bool up = (lo & k) == 0;
                        const int ka = key[lo], kb = key[hi];
                        if ((ka > kb) == up) {
                            key[lo] = kb; key[hi] = ka;
                            const int ma = msk[lo];
                            msk[lo] = msk[hi]; msk[hi] = ma;
                        }
                    }
                    __syncwarp();
                }
            int2* orow = grow + (size_t)g * gcap;
            for (int t = lane; t < cnt; t += 32) {
                const int h = key[t], j0 = gstart[h], nj = gstart[h + 1] - j0;
                orow[t] = make_int2(j0, msk[t] | ((nj - 1) << 16));
                bits += (unsigned long long)__popc(msk[t]);
            }
            if (lane == 0) { glen[g] = cnt; ent += (unsigned long long)cnt; }
        }
        __syncwarp();
        for (int t = lane; t < GH_SLOTS; t += 32) { key[t] = -1; msk[t] = 0; }
        __syncwarp();
    }
    for (int o = 16; o > 0; o >>= 1) {
        ent += __shfl_xor_sync(0xffffffffu, ent, o);
        bits += __shfl_xor_sync(0xffffffffu, bits, o);
    }
    const bool any_over = __any_sync(0xffffffffu, over);
    if (lane == 0) {
        if (ent) atomicAdd(&misc[0], ent);
        if (bits) atomicAdd(&misc[1], bits);
        if (any_over) atomicAdd(&misc[2], 1ull);
    }
}

// The mixed-precision switched energy over the group rows: a warp per group row (the group's atoms
// in registers), a lane per entry (the partner group's atoms gathered as one run of consecutive
// fixed-point positions), the entry's G x G atom pairs evaluated without branches: a pair whose
// mask bit is clear or that lies beyond the cutoff takes r^2 = rc^2, where the switch polynomial is
// exactly 0.  Per entry and row atom the pair terms are summed in FP32 over the entry's (at most G)
// partners, then added to the row atom's float-float Coulomb sum (TwoSum) and FP32 LJ sum, which
// are multiplied by q_i and eps_i at the row's end (factored as in k_energy_list_mix).  Atom
// parameters come from the class table in shared memory, indexed by the class the fixed-point
// mirror carries in w.  G: the largest group size of the system (3 or 4); the next entry's
// positions are loaded while the current one is evaluated.
template <int G, bool ISO, int MINB, bool PF>
__global__ void __launch_bounds__(GE_THREADS, MINB) k_energy_groups(const uint4* __restrict__ fx, const float4* __restrict__ cls,
                                                                    int ncls, const int* __restrict__ gstart, int ngroup,
                                                                    const int2* __restrict__ grow,
                                                                    const int* __restrict__ glen, int gcap, GroupGeom Gm,
                                                                    double* part) {
    extern __shared__ float4 s_cls[];
    for (int c = threadIdx.x; c < ncls; c += blockDim.x) s_cls[c] = cls[c];
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nwarps = (gridDim.x * blockDim.x) >> 5;
    const float c2 = Gm.c2, n2 = Gm.n2, k3 = Gm.k3;
    float EH = 0.0f, EL = 0.0f, VH = 0.0f, VL = 0.0f;
    for (int g = warp; g < ngroup; g += nwarps) {
        const int a0 = gstart[g], ni = gstart[g + 1] - a0;   // 1..G, the same in every lane
        uint4 fi[G];
        float si[G];
#pragma unroll
        for (int a = 0; a < G; a++) {
            fi[a] = fx[a0 + (a < ni ? a : 0)];
            si[a] = s_cls[fi[a].w].w;
        }
        float ch[G], cl[G], vs[G];
#pragma unroll
        for (int a = 0; a < G; a++) { ch[a] = 0.f; cl[a] = 0.f; vs[a] = 0.f; }
        const int m = glen[g];
        const int2* row = grow + (size_t)g * gcap;
        // an entry is (first atom of the partner group, pair mask | (its size - 1) << 16); positions
        // past the partner group's size repeat its first atom (their mask bits are clear)
        int2 e = lane < m ? row[lane] : make_int2(a0, 0);
        uint4 fj[G];
#pragma unroll
        for (int b = 0; b < G; b++) fj[b] = fx[e.x + (b <= (e.y >> 16) ? b : 0)];
        for (int k = lane; k < m; k += 32) {
            const int2 ec = e;
            uint4 fc[G];
#pragma unroll
            for (int b = 0; b < G; b++) fc[b] = fj[b];
            // PF: the next entry's gathers are issued here, in flight while this one is evaluated;
            // otherwise at the end of the iteration
            if (PF) {
                e = k + 32 < m ? row[k + 32] : make_int2(a0, 0);
#pragma unroll
                for (int b = 0; b < G; b++) fj[b] = fx[e.x + (b <= (e.y >> 16) ? b : 0)];
            }
            const int mask = ec.y;
            float4 pj[G];
#pragma unroll
            for (int b = 0; b < G; b++) pj[b] = s_cls[fc[b].w];
#pragma unroll
            for (int a = 0; a < G; a++) {
                if (a >= ni) break;
                float th = 0.f, tl = 0.f, tv = 0.f;
#pragma unroll
                for (int b = 0; b < G; b++) {
                    float r2;
                    if (ISO) {
                        const float ux = __int2float_rn((int)(fc[b].x - fi[a].x)), uy = __int2float_rn((int)(fc[b].y - fi[a].y)),
                                    uz = __int2float_rn((int)(fc[b].z - fi[a].z));
                        const float r2u = fmaf(ux, ux, fmaf(uy, uy, uz * uz));
                        r2 = fmaf(r2u, Gm.L2h, r2u * Gm.L2l);
                    } else {
                        const float dx = fixed_delta(fi[a].x, fc[b].x, Gm.Ls[0], Gm.Ll[0]);
                        const float dy = fixed_delta(fi[a].y, fc[b].y, Gm.Ls[1], Gm.Ll[1]);
                        const float dz = fixed_delta(fi[a].z, fc[b].z, Gm.Ls[2], Gm.Ll[2]);
                        r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
                    }
                    // masked out or beyond rc: r^2 = rc^2, where the switch polynomial is 0
                    r2 = (((mask >> (a * 4 + b)) & 1) && r2 <= c2) ? r2 : c2;
                    float rinv = rsqrtf(r2);
                    rinv = rinv * fmaf(-0.5f * r2 * rinv, rinv, 1.5f);   // one Newton step
                    const float uu = fmaxf(r2, n2);
                    const float aa = c2 - uu;
                    const float f = aa * aa * fmaf(2.0f, uu, k3);
                    const float gg = rinv * f;
                    th = fmaf(pj[b].x, gg, th);
                    tl = fmaf(pj[b].y, gg, tl);
                    const float y = (si[a] + pj[b].w) * rinv;
                    const float x2 = y * y;
                    const float x6 = x2 * x2 * x2;
                    tv = fmaf(pj[b].z, fmaf(x6, x6, -x6) * f, tv);
                }
                float sm, er;
                two_sum(ch[a], th, sm, er);
                ch[a] = sm;
                cl[a] += tl + er;
                vs[a] += tv;
            }
            if (!PF) {
                e = k + 32 < m ? row[k + 32] : make_int2(a0, 0);
#pragma unroll
                for (int b = 0; b < G; b++) fj[b] = fx[e.x + (b <= (e.y >> 16) ? b : 0)];
            }
        }
#pragma unroll
        for (int a = 0; a < G; a++)
            if (a < ni) mix_row_flush(s_cls[fi[a].w], ch[a], cl[a], vs[a], EH, EL, VH, VL);
    }
    block_reduce2(((double)EH + (double)EL) * Gm.inv_f1, ((double)VH + (double)VL) * Gm.inv_f1, part + 2 * blockIdx.x);
}

// The same energy with two entries per lane in packed FP32: entries k and k + 1 of a row take the
// two halves of float2 values, so one sm_100+ packed instruction (add, multiply or FMA on a
// register pair) does the work of both.  The switch is evaluated as P = u^2 (3 D - 2 u) on
// u = clamp(rc^2 - r^2, 0, D), D = rc^2 - ron^2: the reference's polynomial (c2 - r^2)^2
// (c2 + 2 r^2 - 3 n2) rewritten in u, D^3 below ron and 0 beyond rc and for masked pairs (their
// r^2 is set to rc^2).  rc^2 - r^2 is exact in the switching region, the clamps run on the ALU
// pipe, and the block sums take 1 / (that polynomial at u = D) in FP64 at the end (inv_p1).  The
// partner atoms' parameters are read from per-parameter tables in shared memory straight into the
// halves of each float2.  Per entry pair and row atom the terms are summed in FP32, then into the
// row atom's float-float Coulomb sum and FP32 LJ sum as in k_energy_groups.
//
// Placement: a row of G atoms whose offsets from its first atom stay within emax (each component)
// places the partner atoms relative to that first atom (one fixed-point difference and conversion
// per partner atom, not per atom pair) and adds each row atom's own offset; every partner within
// rc is then at its minimum image.  Other rows (fewer atoms, or wider than emax in small boxes)
// take the per-pair fixed-point displacement, exact at any box size.  The choice is made once per
// row and is the same in every lane.
__device__ __forceinline__ float2 pk_add(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 pk_mul(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 pk_fma(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ float2 pk_dup(float a) { return make_float2(a, a); }

// fixed-point displacements of two partner coordinates from base, in Angstrom (float-float scale)
__device__ __forceinline__ float2 pk_delta(uint32_t base, uint32_t xa, uint32_t xb, float2 Lh, float2 Ll) {
    const float2 f = make_float2(__int2float_rn((int)(xa - base)), __int2float_rn((int)(xb - base)));
    return pk_fma(f, Lh, pk_mul(f, Ll));
}

// The constants of the packed kernel, each duplicated into both halves of a float2
struct PkConst {
    float2 Lh[3], Ll[3];     // box / 2^32 per axis, float-float
    float2 c2, m1, m2, d3, m3;
    float c2s, D;
};

__device__ __forceinline__ PkConst pk_const(const GroupGeom& G) {
    PkConst K;
    for (int k = 0; k < 3; k++) { K.Lh[k] = make_float2(G.Ls[k], G.Ls[k]); K.Ll[k] = make_float2(G.Ll[k], G.Ll[k]); }
    K.c2 = make_float2(G.c2, G.c2);
    K.m1 = make_float2(-1.0f, -1.0f);
    K.m2 = make_float2(-2.0f, -2.0f);
    K.d3 = make_float2(3.0f * G.D, 3.0f * G.D);
    K.m3 = make_float2(-3.0f, -3.0f);
    K.c2s = G.c2;
    K.D = G.D;
    return K;
}

// The pair terms of one row atom with one partner atom in entries A and B (inA / inB: the pair is
// in the rows), added to the row atom's per-entry sums.
__device__ __forceinline__ void pk_slot(float2 dx, float2 dy, float2 dz, bool inA, bool inB, float2 si, float2 qh,
                                        float2 ql, float2 ep, float2 sg, const PkConst& K, float2& tc, float2& tl,
                                        float2& tv) {
    float2 r2 = pk_fma(dx, dx, pk_fma(dy, dy, pk_mul(dz, dz)));
    r2.x = inA ? r2.x : K.c2s;
    r2.y = inB ? r2.y : K.c2s;
    const float2 d = pk_fma(r2, K.m1, K.c2);                                   // rc^2 - r^2
    const float2 u = make_float2(fminf(fmaxf(d.x, 0.0f), K.D), fminf(fmaxf(d.y, 0.0f), K.D));
    const float2 sw = pk_mul(pk_mul(u, u), pk_fma(u, K.m2, K.d3));             // D^3 S
    float2 ri = make_float2(rsqrtf(r2.x), rsqrtf(r2.y));
    // one Newton step, scaled by -2 (exact): ri = -2 / r.  The Coulomb sums carry the factor (the
    // row's flush takes it out), the half sigmas carry -1/2 (the per-parameter table holds them so)
    ri = pk_mul(ri, pk_fma(pk_mul(r2, ri), ri, K.m3));
    const float2 gg = pk_mul(ri, sw);
    tc = pk_fma(qh, gg, tc);
    tl = pk_fma(ql, gg, tl);
    const float2 y = pk_mul(pk_add(si, sg), ri);
    const float2 x2 = pk_mul(y, y);
    const float2 x6 = pk_mul(pk_mul(x2, x2), x2);
    tv = pk_fma(ep, pk_mul(pk_fma(x6, x6, make_float2(-x6.x, -x6.y)), sw), tv);   // the negation folds into the FMA
}

// The row state of the packed kernels: the row atoms' offsets from the first (negated, duplicated
// into both halves), their half sigmas, raw positions (per-pair placement) and the per-atom sums.
template <int G>
struct PkRow {
    uint4 f0;
    uint4 fi[G];
    float2 nox[G], noy[G], noz[G], si[G];
    float ch[G], cl[G], vs[G];
    int a0, ni;
    bool fast;
};

template <int G>
__device__ __forceinline__ void pk_row_begin(PkRow<G>& R, const uint4* __restrict__ fx, const float* s_sg, int a0, int ni,
                                             const GroupGeom& Gm) {
    R.a0 = a0;
    R.ni = ni;
    R.f0 = fx[a0];
    float off = 0.0f;
#pragma unroll
    for (int a = 0; a < G; a++) {
        const uint4 fa = fx[a0 + (a < ni ? a : 0)];
        R.fi[a] = fa;
        const float ox = fixed_delta(R.f0.x, fa.x, Gm.Ls[0], Gm.Ll[0]);
        const float oy = fixed_delta(R.f0.y, fa.y, Gm.Ls[1], Gm.Ll[1]);
        const float oz = fixed_delta(R.f0.z, fa.z, Gm.Ls[2], Gm.Ll[2]);
        R.nox[a] = pk_dup(-ox);
        R.noy[a] = pk_dup(-oy);
        R.noz[a] = pk_dup(-oz);
        off = fmaxf(off, fmaxf(fabsf(ox), fmaxf(fabsf(oy), fabsf(oz))));
        R.si[a] = pk_dup(s_sg[fa.w]);
        R.ch[a] = 0.f;
        R.cl[a] = 0.f;
        R.vs[a] = 0.f;
    }
    R.fast = ni == G && off <= Gm.emax;   // the same in every lane
}

template <int G>
__device__ __forceinline__ void pk_row_end(const PkRow<G>& R, const uint4* __restrict__ fx, const float4* s_cls, float& EH,
                                           float& EL, float& VH, float& VL) {
#pragma unroll
    for (int a = 0; a < G; a++)
        if (a < R.ni) mix_row_flush(s_cls[fx[R.a0 + a].w], -0.5f * R.ch[a], -0.5f * R.cl[a], R.vs[a], EH, EL, VH, VL);
}

// FP32 sums of a row atom's pair terms over one item (both halves), before they go into the row's
// float-float Coulomb and FP32 LJ sums (summing two items before that moved the Coulomb total of a
// 550-water box 2.7e-7 from the per-atom list kernel's, past their 2e-7 agreement)
template <int G>
struct PkAcc {
    float2 tc[G], tl[G], tv[G];
    __device__ __forceinline__ void zero() {
#pragma unroll
        for (int a = 0; a < G; a++) { tc[a] = pk_dup(0.f); tl[a] = pk_dup(0.f); tv[a] = pk_dup(0.f); }
    }
};

// the item sums into the row sums (the atoms past the row's size hold zeros)
template <int G>
__device__ __forceinline__ void pk_flush(PkRow<G>& R, PkAcc<G>& T) {
#pragma unroll
    for (int a = 0; a < G; a++) {
        float sm, er;
        two_sum(R.ch[a], T.tc[a].x + T.tc[a].y, sm, er);
        R.ch[a] = sm;
        R.cl[a] += (T.tl[a].x + T.tl[a].y) + er;
        R.vs[a] += T.tv[a].x + T.tv[a].y;
    }
    T.zero();
}

// One item: entries A and B (their G partner atoms fA, fB and masks mA, mB) against the row's atoms,
// added to T.  FAST: relative placement, all G row atoms, no per-slot branch; else per-pair
// displacement.
template <int G, bool FAST>
__device__ __forceinline__ void pk_item(PkRow<G>& R, const uint4 (&fA)[G], const uint4 (&fB)[G], int mA, int mB,
                                        const float* s_qh, const float* s_ql, const float* s_ep, const float* s_sg,
                                        const PkConst& K, PkAcc<G>& T) {
#pragma unroll
    for (int b = 0; b < G; b++) {
        const int cA = fA[b].w, cB = fB[b].w;
        const float2 qh = make_float2(s_qh[cA], s_qh[cB]), ql = make_float2(s_ql[cA], s_ql[cB]);
        const float2 ep = make_float2(s_ep[cA], s_ep[cB]), sg = make_float2(s_sg[cA], s_sg[cB]);
        float2 jx, jy, jz;
        if (FAST) {
            jx = pk_delta(R.f0.x, fA[b].x, fB[b].x, K.Lh[0], K.Ll[0]);
            jy = pk_delta(R.f0.y, fA[b].y, fB[b].y, K.Lh[1], K.Ll[1]);
            jz = pk_delta(R.f0.z, fA[b].z, fB[b].z, K.Lh[2], K.Ll[2]);
        }
#pragma unroll
        for (int a = 0; a < G; a++) {
            if (!FAST && a >= R.ni) break;
            float2 dx, dy, dz;
            if (FAST) {
                if (a == 0) { dx = jx; dy = jy; dz = jz; }
                else { dx = pk_add(jx, R.nox[a]); dy = pk_add(jy, R.noy[a]); dz = pk_add(jz, R.noz[a]); }
            } else {
                dx = pk_delta(R.fi[a].x, fA[b].x, fB[b].x, K.Lh[0], K.Ll[0]);
                dy = pk_delta(R.fi[a].y, fA[b].y, fB[b].y, K.Lh[1], K.Ll[1]);
                dz = pk_delta(R.fi[a].z, fA[b].z, fB[b].z, K.Lh[2], K.Ll[2]);
            }
            const int bit = 1 << (a * 4 + b);
            pk_slot(dx, dy, dz, (mA & bit) != 0, (mB & bit) != 0, R.si[a], qh, ql, ep, sg, K, T.tc[a], T.tl[a], T.tv[a]);
        }
    }
}

// the class table and its per-parameter copies in shared memory (the packed kernels' layout; the
// half sigmas times -1/2, the scale of pk_slot's inverse distance)
__device__ __forceinline__ void pk_load_classes(const float4* __restrict__ cls, int ncls, float4* s_cls) {
    float* s_qh = (float*)(s_cls + ncls);
    for (int c = threadIdx.x; c < ncls; c += blockDim.x) {
        const float4 v = cls[c];
        s_cls[c] = v;
        s_qh[c] = v.x; s_qh[ncls + c] = v.y; s_qh[2 * ncls + c] = v.z; s_qh[3 * ncls + c] = -0.5f * v.w;
    }
}

// Packed kernel, gathers in registers: a warp per row, entries k and k + 1 per lane.
template <int G, int NT, int MINB>
__global__ void __launch_bounds__(NT, MINB) k_energy_groups_x2(const uint4* __restrict__ fx, const float4* __restrict__ cls,
                                                               int ncls, const int* __restrict__ gstart, int ngroup,
                                                               const int2* __restrict__ grow, const int* __restrict__ glen,
                                                               int gcap, GroupGeom Gm, double* part) {
    extern __shared__ float4 s_cls[];
    pk_load_classes(cls, ncls, s_cls);
    const float* s_qh = (const float*)(s_cls + ncls);
    const float *s_ql = s_qh + ncls, *s_ep = s_ql + ncls, *s_sg = s_ep + ncls;
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nwarps = (gridDim.x * blockDim.x) >> 5;
    const PkConst K = pk_const(Gm);
    float EH = 0.0f, EL = 0.0f, VH = 0.0f, VL = 0.0f;
    PkRow<G> R;
    for (int g = warp; g < ngroup; g += nwarps) {
        const int a0 = gstart[g];
        pk_row_begin(R, fx, s_sg, a0, gstart[g + 1] - a0, Gm);
        const int m = glen[g];
        const int2* row = grow + (size_t)g * gcap;
        auto sweep = [&](auto fast_tag) {
            constexpr bool FAST = decltype(fast_tag)::value;
            PkAcc<G> T;
            T.zero();
            for (int k = 2 * lane; k < m; k += 64) {
                // entries k and k + 1 (past the row's end: the row group itself, all mask bits clear)
                const int2 eA = row[k];
                const int2 eB = k + 1 < m ? row[k + 1] : make_int2(a0, 0);
                uint4 fA[G], fB[G];
#pragma unroll
                for (int b = 0; b < G; b++) {
                    fA[b] = fx[eA.x + (b <= (eA.y >> 16) ? b : 0)];
                    fB[b] = fx[eB.x + (b <= (eB.y >> 16) ? b : 0)];
                }
                pk_item<G, FAST>(R, fA, fB, eA.y, eB.y, s_qh, s_ql, s_ep, s_sg, K, T);
                pk_flush(R, T);
            }
        };
        if (R.fast) sweep(std::true_type{});
        else sweep(std::false_type{});
        pk_row_end(R, fx, s_cls, EH, EL, VH, VL);
    }
    block_reduce2(((double)EH + (double)EL) * Gm.inv_p1, ((double)VH + (double)VL) * Gm.inv_p1, part + 2 * blockIdx.x);
}

// Packed kernel, gathers prefetched in registers: a warp's items (row after row, entries k and
// k + 1 of a row per lane, the same sequence in every lane) with the next item's 2G partner atoms
// loaded into a second register set while the current item is evaluated, and each item's entries
// loaded two items ahead (unchecked: checked against the row's length when its atoms are loaded,
// by which time that length has arrived).  The loop body is written twice, so the two register
// sets swap roles without copies.  A row's sums are flushed when the next item belongs to another
// row.  It pays when the rows stream from DRAM; with the rows resident in L2 the plain packed
// kernel is faster (fewer instructions).
template <int G, int NT, int MINB>
__global__ void __launch_bounds__(NT, MINB) k_energy_groups_x2r(const uint4* __restrict__ fx, const float4* __restrict__ cls,
                                                                int ncls, const int* __restrict__ gstart, int ngroup,
                                                                const int2* __restrict__ grow, const int* __restrict__ glen,
                                                                int gcap, GroupGeom Gm, double* part) {
    extern __shared__ float4 s_cls[];
    pk_load_classes(cls, ncls, s_cls);
    const float* s_qh = (const float*)(s_cls + ncls);
    const float *s_ql = s_qh + ncls, *s_ep = s_ql + ncls, *s_sg = s_ep + ncls;
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nwarps = (gridDim.x * blockDim.x) >> 5;
    const PkConst K = pk_const(Gm);
    struct Cur { int g, a0, m, k; };
    auto advance = [&](Cur& c) {
        if (c.k - 2 * lane + 64 < c.m) {
            c.k += 64;
        } else {
            c.g += nwarps;
            c.k = 2 * lane;
            if (c.g < ngroup) { c.a0 = gstart[c.g]; c.m = glen[c.g]; }
        }
    };
    auto raw = [&](const Cur& c, int2& A, int2& B) {
        A = make_int2(0, 0);
        B = make_int2(0, 0);
        if (c.g < ngroup) {
            const int2* r = grow + (size_t)c.g * gcap;
            A = r[min(c.k, gcap - 1)];
            B = r[min(c.k + 1, gcap - 1)];
        }
    };
    auto gather = [&](const Cur& c, int2& A, int2& B, uint4 (&fA)[G], uint4 (&fB)[G]) {
        if (c.g < ngroup) {
            if (!(c.k < c.m)) A = make_int2(c.a0, 0);   // past the row's end: the row group, no mask bits
            if (!(c.k + 1 < c.m)) B = make_int2(c.a0, 0);
#pragma unroll
            for (int b = 0; b < G; b++) {
                fA[b] = fx[A.x + (b <= (A.y >> 16) ? b : 0)];
                fB[b] = fx[B.x + (b <= (B.y >> 16) ? b : 0)];
            }
        }
    };
    float EH = 0.0f, EL = 0.0f, VH = 0.0f, VL = 0.0f;
    PkRow<G> R;
    PkAcc<G> T;
    T.zero();
    int rg = -1;
    Cur c0{warp, 0, 0, 2 * lane};
    if (c0.g < ngroup) { c0.a0 = gstart[c0.g]; c0.m = glen[c0.g]; }
    int2 A0, B0, A1, B1;
    uint4 fA0[G], fB0[G], fA1[G], fB1[G];
    raw(c0, A0, B0);
    gather(c0, A0, B0, fA0, fB0);
    Cur c1 = c0;
    advance(c1);
    raw(c1, A1, B1);
    // one item: c (its atoms fA, fB already loaded); cn, An, Bn: the next item, whose atoms go to gA, gB
    auto step = [&](Cur& c, int2& A, int2& B, uint4 (&fA)[G], uint4 (&fB)[G], Cur& cn, int2& An, int2& Bn,
                    uint4 (&gA)[G], uint4 (&gB)[G]) {
        Cur c2 = cn;
        advance(c2);
        int2 A2, B2;
        raw(c2, A2, B2);
        gather(cn, An, Bn, gA, gB);
        if (c.g != rg) {
            if (rg >= 0) pk_row_end(R, fx, s_cls, EH, EL, VH, VL);
            pk_row_begin(R, fx, s_sg, c.a0, gstart[c.g + 1] - c.a0, Gm);
            rg = c.g;
        }
        if (R.fast) pk_item<G, true>(R, fA, fB, A.y, B.y, s_qh, s_ql, s_ep, s_sg, K, T);
        else pk_item<G, false>(R, fA, fB, A.y, B.y, s_qh, s_ql, s_ep, s_sg, K, T);
        pk_flush(R, T);
        c = c2;          // the item after next takes this item's cursor and entries
        A = A2;
        B = B2;
    };
    while (true) {
        if (c0.g >= ngroup) break;
        step(c0, A0, B0, fA0, fB0, c1, A1, B1, fA1, fB1);   // c0 <- item after c1
        if (c1.g >= ngroup) break;
        step(c1, A1, B1, fA1, fB1, c0, A0, B0, fA0, fB0);   // c1 <- item after c0
    }
    if (rg >= 0) pk_row_end(R, fx, s_cls, EH, EL, VH, VL);
    block_reduce2(((double)EH + (double)EL) * Gm.inv_p1, ((double)VH + (double)VL) * Gm.inv_p1, part + 2 * blockIdx.x);
}

template <typename T>
static int galloc(T** p, size_t count) {
    cudaError_t e = cudaMalloc((void**)p, std::max<size_t>(1, count) * sizeof(T));
    if (e != cudaSuccess) { *p = nullptr; return fail(MCG_ECUDA, std::string("cudaMalloc: ") + cudaGetErrorString(e)); }
    return MCG_OK;
}

void GroupPairs::release() {
    void* p[] = {d_gstart, d_gof, d_grow, d_glen, d_misc};
    for (void* q : p) if (q) cudaFree(q);
    d_gstart = d_gof = d_glen = nullptr;
    d_grow = nullptr;
    d_misc = nullptr;
    grow_cap = 0;
}

int GroupPairs::setup(const std::vector<int>& resid) {
    release();
    ok = false;
    n = (int)resid.size();
    std::vector<int> gs, gof(n);
    for (int i = 0; i < n; i++) {
        if (i == 0 || resid[i] != resid[i - 1] || i - gs.back() == 4) gs.push_back(i);
        gof[i] = (int)gs.size() - 1;
    }
    ngroup = (int)gs.size();
    gs.push_back(n);
    gmax = 1;
    for (int g = 0; g < ngroup; g++) gmax = std::max(gmax, gs[g + 1] - gs[g]);
    int rc;
    if ((rc = galloc(&d_gstart, gs.size())) || (rc = galloc(&d_gof, (size_t)n)) || (rc = galloc(&d_glen, (size_t)ngroup)) ||
        (rc = galloc(&d_misc, 3)))
        return rc;
    GK(cudaMemcpy(d_gstart, gs.data(), sizeof(int) * gs.size(), cudaMemcpyHostToDevice));
    GK(cudaMemcpy(d_gof, gof.data(), sizeof(int) * n, cudaMemcpyHostToDevice));
    return MCG_OK;
}

int GroupPairs::build(cudaStream_t st, const int* rows, const int* lens, int cap) {
    ok = false;
    if (!d_gstart) return fail(MCG_EINVAL, "group pairs used before setup");
    gcap = std::min(cap, GH_MAX);
    const size_t need = (size_t)ngroup * gcap;
    if (need > grow_cap) {
        if (d_grow) cudaFree(d_grow);
        d_grow = nullptr;
        grow_cap = 0;
        int rc = galloc(&d_grow, need);
        if (rc) return rc;
        grow_cap = need;
    }
    GK(cudaMemsetAsync(d_misc, 0, 3 * sizeof(unsigned long long), st));
    const int blocks = std::min((ngroup + GB_WARPS - 1) / GB_WARPS, 152 * 16);
    k_group_rows<<<blocks, GB_WARPS * 32, 0, st>>>(d_gstart, d_gof, ngroup, rows, lens, cap, d_grow, d_glen, gcap, d_misc);
    GK(cudaGetLastError());
    unsigned long long misc[3];
    GK(cudaMemcpyAsync(misc, d_misc, sizeof misc, cudaMemcpyDeviceToHost, st));
    GK(cudaStreamSynchronize(st));
    build_launches += 1;
    nentries = (int64_t)misc[0];
    nbits = (int64_t)misc[1];
    if (misc[2]) return fail(MCG_ECAPACITY, "a group row has more partner groups than the group-pair build holds");
    ok = true;
    return MCG_OK;
}

int GroupPairs::launch_energy(cudaStream_t st, int v, const uint4* fx, const float4* cls, int ncls, const GroupGeom& G,
                              double* part) {
    const size_t smem = sizeof(float4) * (size_t)ncls;
    int blocks = 0;
#define MCG_GROUP_ONE(GS_, ISO_, B_, PF_)                                                                        \
    blocks = 152 * B_;                                                                                            \
    k_energy_groups<GS_, ISO_, B_, PF_><<<blocks, GE_THREADS, smem, st>>>(fx, cls, ncls, d_gstart, ngroup, d_grow, d_glen, \
                                                                          gcap, G, part);
#define MCG_GROUP_X2(GS_, NT_, B_)                                                                                \
    blocks = 152 * B_;                                                                                            \
    k_energy_groups_x2<GS_, NT_, B_><<<blocks, NT_, 2 * smem, st>>>(fx, cls, ncls, d_gstart, ngroup, d_grow, d_glen, gcap, \
                                                                G, part);
#define MCG_GROUP_X2R(GS_, NT_, B_)                                                                               \
    blocks = 152 * B_;                                                                                            \
    k_energy_groups_x2r<GS_, NT_, B_><<<blocks, NT_, 2 * smem, st>>>(fx, cls, ncls, d_gstart, ngroup, d_grow, d_glen, \
                                                                     gcap, G, part);
#define MCG_GROUP_G(GS_)                                                                                          \
    if (v == 0) { if (G.iso) { MCG_GROUP_ONE(GS_, true, 2, true) } else { MCG_GROUP_ONE(GS_, false, 2, true) } }   \
    else if (v == 1) { if (G.iso) { MCG_GROUP_ONE(GS_, true, 3, false) } else { MCG_GROUP_ONE(GS_, false, 3, false) } } \
    else if (v == 2) { MCG_GROUP_X2(GS_, 256, 2) }                                                                 \
    else { MCG_GROUP_X2R(GS_, 128, 3) }
    if (gmax <= 3) { MCG_GROUP_G(3) } else { MCG_GROUP_G(4) }
#undef MCG_GROUP_G
#undef MCG_GROUP_X2R
#undef MCG_GROUP_X2
#undef MCG_GROUP_ONE
    return blocks;
}

}  // namespace mcg
