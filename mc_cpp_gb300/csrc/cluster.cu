// Cluster-pair list and the cluster-pair mixed-precision switched energy (periodic boxes).
//
// Build (once per Verlet build, after the rows):
//   k_col_assign   column (x-y cell) of every atom from its fixed-point position
//   k_col_scan     exclusive scans of the column sizes and of the clusters per column
//   k_col_scatter  atoms into their columns
//   k_col_sort     each column sorted along z (bitonic, shared memory), cut into clusters of 8
//   k_cluster_pairs  per cluster A: the clusters B holding a Verlet partner of one of A's atoms and
//                  owned by A, as a sorted list with the 64-bit mask of the Verlet pairs between
//                  the two clusters (bitmap of B in shared memory, rank by popcount)
// Per energy call:
//   k_cluster_pack   slot offsets from the cluster's first atom (exact fixed-point difference,
//                  scaled to FP32), parameters, and each cluster's bounding box
//   k_energy_cluster warp per i-cluster (taken from a work counter), 8 x 8 slot pairs per
//                  cluster pair in two passes of 32 lanes; cluster pairs whose boxes are farther
//                  apart than rc are skipped; one FP64 partial pair per cluster, summed in a fixed
//                  order by k_finalize.
//
// The pair terms are those of FField_MDBAS::computeNonBonded_switch (FField_MDBAS.cpp:336-424):
// r^2 <= rc^2 in the list, switch S(r^2) = (rc^2-r^2)^2 (rc^2+2r^2-3ron^2)/(rc^2-ron^2)^3 above
// ron^2, Coulomb q_i q_j / r and LJ eps_i eps_j (x^12 - x^6), x = (sig_i + sig_j) / r, unscaled.
#include <algorithm>
#include <cmath>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "cluster.hpp"
#include "engine.hpp"
#include "pair_math.cuh"

namespace mcg {

#define CKC(call)                                                                              \
    do {                                                                                       \
        cudaError_t e_ = (call);                                                               \
        if (e_ != cudaSuccess) return fail(MCG_ECUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

constexpr int CL = 8;                  // atoms per cluster
constexpr int COL_SORT_MAX = 16384;    // largest column sorted in shared memory (128 KiB of keys)
constexpr int PAIR_SMEM_MAX = 200 * 1024;

// ---- build --------------------------------------------------------------------------------
__device__ __forceinline__ unsigned fixed_cell(uint32_t f, int nc) {
    // fixed-point coordinate (wrapped position / L * 2^32, signed) -> cell in [0, nc)
    return (unsigned)(((unsigned long long)(f ^ 0x80000000u) * (unsigned)nc) >> 32);
}

__global__ void k_col_assign(const uint4* __restrict__ fx, int n, int ncx, int ncy, int* col_of, int* col_count) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint4 f = fx[i];
    const int c = (int)fixed_cell(f.x, ncx) + ncx * (int)fixed_cell(f.y, ncy);
    col_of[i] = c;
    atomicAdd(&col_count[c], 1);
}

// One block: col_start = exclusive scan of the column sizes, ccl_start = of the clusters per
// column; both get their total at [ncol]; misc[0] = the largest column.
__global__ void k_col_scan(const int* __restrict__ col_count, int ncol, int* col_start, int* ccl_start, int* col_fill,
                           unsigned long long* misc) {
    __shared__ int sa[1024], sb[1024];
    __shared__ int ca, cb, mx;
    if (threadIdx.x == 0) { ca = 0; cb = 0; mx = 0; }
    __syncthreads();
    for (int base = 0; base < ncol; base += 1024) {
        const int i = base + threadIdx.x;
        const int v = i < ncol ? col_count[i] : 0;
        const int w = (v + CL - 1) / CL;
        sa[threadIdx.x] = v;
        sb[threadIdx.x] = w;
        if (v > 0) atomicMax(&mx, v);
        __syncthreads();
        for (int o = 1; o < 1024; o <<= 1) {
            const int ta = threadIdx.x >= o ? sa[threadIdx.x - o] : 0;
            const int tb = threadIdx.x >= o ? sb[threadIdx.x - o] : 0;
            __syncthreads();
            sa[threadIdx.x] += ta;
            sb[threadIdx.x] += tb;
            __syncthreads();
        }
        if (i < ncol) { col_start[i] = ca + sa[threadIdx.x] - v; ccl_start[i] = cb + sb[threadIdx.x] - w; col_fill[i] = 0; }
        __syncthreads();
        if (threadIdx.x == 1023) { ca += sa[1023]; cb += sb[1023]; }
        __syncthreads();
    }
    if (threadIdx.x == 0) { col_start[ncol] = ca; ccl_start[ncol] = cb; misc[0] = (unsigned long long)mx; }
}

__global__ void k_col_scatter(const int* __restrict__ col_of, int n, const int* __restrict__ col_start, int* col_fill,
                              int* col_atoms) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int c = col_of[i];
    col_atoms[col_start[c] + atomicAdd(&col_fill[c], 1)] = i;
}

// One block per column: sort by (z, atom index) and cut into clusters of 8 (padding slots -1).
__global__ void k_col_sort(const uint4* __restrict__ fx, const int* __restrict__ col_start, const int* __restrict__ ccl_start,
                           const int* __restrict__ col_atoms, int* cl_atom, int* cl_of) {
    extern __shared__ unsigned long long keys[];
    const int c = blockIdx.x;
    const int b = col_start[c], m = col_start[c + 1] - b;
    if (m == 0) return;
    int m2 = 1;
    while (m2 < m) m2 <<= 1;
    for (int t = threadIdx.x; t < m2; t += blockDim.x) {
        unsigned long long k = ~0ull;
        if (t < m) {
            const int a = col_atoms[b + t];
            k = ((unsigned long long)(fx[a].z ^ 0x80000000u) << 32) | (unsigned)a;
        }
        keys[t] = k;
    }
    __syncthreads();
    for (int k = 2; k <= m2; k <<= 1)
        for (int j = k >> 1; j > 0; j >>= 1) {
            for (int t = threadIdx.x; t < m2; t += blockDim.x) {
                const int l = t ^ j;
                if (l > t) {
                    const bool up = (t & k) == 0;
                    const unsigned long long x = keys[t], y = keys[l];
                    if ((x > y) == up) { keys[t] = y; keys[l] = x; }
                }
            }
            __syncthreads();
        }
    const int c0 = ccl_start[c];
    const int mp = (m + CL - 1) / CL * CL;
    for (int t = threadIdx.x; t < mp; t += blockDim.x) {
        const int slot = c0 * CL + t;
        if (t < m) {
            const int a = (int)(unsigned)(keys[t] & 0xffffffffull);
            cl_atom[slot] = a;
            cl_of[a] = slot;
        } else {
            cl_atom[slot] = -1;
        }
    }
}

// Which of two distinct clusters owns their pair: the lower index when the sum is even, the
// higher when it is odd, so each cluster owns about half of its neighbours.
__device__ __forceinline__ bool owns(int A, int B) { return (A < B) == (((A ^ B) & 1) == 0); }

// One block per cluster A.  Shared memory: bitmap[nwords], wpre[nwords], masks[2 * capP].
__global__ void __launch_bounds__(256) k_cluster_pairs(const int* __restrict__ cl_atom, const int* __restrict__ cl_of,
                                                       const int* __restrict__ nbr, const int* __restrict__ nup,
                                                       const int* __restrict__ nlo, int cap, int nwords, int capP,
                                                       int* cp_count, int4* cpl, unsigned long long* misc) {
    extern __shared__ unsigned smem[];
    unsigned* bitmap = smem;
    int* wpre = (int*)(smem + nwords);
    unsigned* masks = smem + 2 * nwords;
    __shared__ int s_scan[256];
    const int A = blockIdx.x;
    const int tid = threadIdx.x, nt = blockDim.x;
    for (int w = tid; w < nwords; w += nt) bitmap[w] = 0u;
    __syncthreads();
    // pass 1: the owned partner clusters
    for (int a = 0; a < CL; a++) {
        const int i = cl_atom[A * CL + a];
        if (i < 0) continue;
        const int up = nup[i], tot = up + nlo[i];
        const int* row = nbr + (size_t)i * cap;
        for (int k = tid; k < tot; k += nt) {
            const int j = k < up ? row[k] : row[cap - 1 - (k - up)];
            const int B = cl_of[j] / CL;
            if (B == A ? j > i : owns(A, B)) atomicOr(&bitmap[B >> 5], 1u << (B & 31));
        }
    }
    __syncthreads();
    // rank of every word: block scan of per-thread chunk counts
    const int per = (nwords + nt - 1) / nt;
    const int w0 = min(nwords, tid * per), w1 = min(nwords, w0 + per);
    int cnt = 0;
    for (int w = w0; w < w1; w++) cnt += __popc(bitmap[w]);
    s_scan[tid] = cnt;
    __syncthreads();
    for (int o = 1; o < nt; o <<= 1) {
        const int t = tid >= o ? s_scan[tid - o] : 0;
        __syncthreads();
        s_scan[tid] += t;
        __syncthreads();
    }
    const int m = s_scan[nt - 1];
    {
        int run = s_scan[tid] - cnt;
        for (int w = w0; w < w1; w++) { wpre[w] = run; run += __popc(bitmap[w]); }
    }
    if (m > capP) {
        if (tid == 0) { atomicMax(&misc[1], (unsigned long long)m); cp_count[A] = 0; }
        return;
    }
    for (int t = tid; t < 2 * m; t += nt) masks[t] = 0u;
    __syncthreads();
    // pass 2: the mask bit (j slot * 8 + i slot) of every owned Verlet pair
    for (int a = 0; a < CL; a++) {
        const int i = cl_atom[A * CL + a];
        if (i < 0) continue;
        const int up = nup[i], tot = up + nlo[i];
        const int* row = nbr + (size_t)i * cap;
        for (int k = tid; k < tot; k += nt) {
            const int j = k < up ? row[k] : row[cap - 1 - (k - up)];
            const int s = cl_of[j];
            const int B = s / CL;
            if (B == A ? j > i : owns(A, B)) {
                const int pos = wpre[B >> 5] + __popc(bitmap[B >> 5] & ((1u << (B & 31)) - 1u));
                const int bit = (s % CL) * CL + a;
                atomicOr(&masks[2 * pos + (bit >> 5)], 1u << (bit & 31));
            }
        }
    }
    __syncthreads();
    unsigned long long bits = 0;
    for (int w = tid; w < nwords; w += nt) {
        unsigned v = bitmap[w];
        int p = wpre[w];
        while (v) {
            const int b = __ffs(v) - 1;
            v &= v - 1u;
            const unsigned lo = masks[2 * p], hi = masks[2 * p + 1];
            cpl[(size_t)A * capP + p] = make_int4(w * 32 + b, (int)lo, (int)hi, 0);
            bits += (unsigned long long)(__popc(lo) + __popc(hi));
            p++;
        }
    }
    for (int o = 16; o > 0; o >>= 1) bits += __shfl_xor_sync(0xffffffffu, bits, o);
    if ((tid & 31) == 0 && bits) atomicAdd(&misc[2], bits);
    if (tid == 0) {
        cp_count[A] = m;
        atomicAdd(&misc[3], (unsigned long long)m);
    }
}

// ---- per energy call ------------------------------------------------------------------------
// Thread per slot: offset of the slot's atom from the cluster's first atom (exact fixed-point
// difference scaled to FP32) with q hi, then (q lo, eps, sig): two float4 per slot, so a cluster's
// slot data is 256 contiguous bytes; the cluster's box and its two half boxes.
__global__ void __launch_bounds__(256) k_cluster_pack(const uint4* __restrict__ fx, const float4* __restrict__ prmf,
                                                      const int* __restrict__ cl_atom, int ncl, ClusterGeom G,
                                                      uint4* cref, float4* cctr, float4* chalf, float4* sdat,
                                                      float4* hbox, int* work) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    const bool in = s < ncl * CL;
    const int A = s / CL;
    const int atom = in ? cl_atom[s] : -1;
    uint4 fr = make_uint4(0, 0, 0, 0);
    if (in) fr = fx[cl_atom[A * CL]];
    float o[3] = {0.f, 0.f, 0.f};
    float mn[3], mx[3];
    if (atom >= 0) {
        const uint4 f = fx[atom];
        o[0] = fixed_delta(fr.x, f.x, G.Ls[0], G.Ll[0]);
        o[1] = fixed_delta(fr.y, f.y, G.Ls[1], G.Ll[1]);
        o[2] = fixed_delta(fr.z, f.z, G.Ls[2], G.Ll[2]);
        const float4 p = prmf[atom];                  // (q hi, q lo, eps, sig)
        sdat[2 * s] = make_float4(o[0], o[1], o[2], p.x);
        sdat[2 * s + 1] = make_float4(p.y, p.z, p.w, 0.f);
    } else if (in) {
        sdat[2 * s] = make_float4(0.f, 0.f, 0.f, 0.f);
        sdat[2 * s + 1] = make_float4(0.f, 0.f, 0.f, 0.f);
    }
    // boxes of the half clusters (slots 0-3, 4-7; reductions over 4 lanes), then of the cluster
    float hmn[3], hmx[3];
#pragma unroll
    for (int k = 0; k < 3; k++) {
        hmn[k] = atom >= 0 ? o[k] : 3.0e38f;
        hmx[k] = atom >= 0 ? o[k] : -3.0e38f;
#pragma unroll
        for (int d = 1; d < CL / 2; d <<= 1) {
            hmn[k] = fminf(hmn[k], __shfl_xor_sync(0xffffffffu, hmn[k], d));
            hmx[k] = fmaxf(hmx[k], __shfl_xor_sync(0xffffffffu, hmx[k], d));
        }
        mn[k] = fminf(hmn[k], __shfl_xor_sync(0xffffffffu, hmn[k], CL / 2));
        mx[k] = fmaxf(hmx[k], __shfl_xor_sync(0xffffffffu, hmx[k], CL / 2));
    }
    if (in && (s % (CL / 2)) == 0) {
        // an empty half (all padding) gets a negative extent: never within range, never wide
        const bool empty = hmn[0] > hmx[0];
        hbox[2 * (s / (CL / 2))] = empty ? make_float4(0.f, 0.f, 0.f, 0.f)
                                         : make_float4(0.5f * (hmn[0] + hmx[0]), 0.5f * (hmn[1] + hmx[1]),
                                                       0.5f * (hmn[2] + hmx[2]), 0.f);
        hbox[2 * (s / (CL / 2)) + 1] = empty ? make_float4(-1.0e30f, -1.0e30f, -1.0e30f, 0.f)
                                             : make_float4(0.5f * (hmx[0] - hmn[0]), 0.5f * (hmx[1] - hmn[1]),
                                                           0.5f * (hmx[2] - hmn[2]), 0.f);
    }
    if (in && (s % CL) == 0) {
        cref[A] = make_uint4(fr.x, fr.y, fr.z, 0u);
        cctr[A] = make_float4(0.5f * (mn[0] + mx[0]), 0.5f * (mn[1] + mx[1]), 0.5f * (mn[2] + mx[2]), 0.f);
        chalf[A] = make_float4(0.5f * (mx[0] - mn[0]), 0.5f * (mx[1] - mn[1]), 0.5f * (mx[2] - mn[2]), 0.f);
    }
    if (s == 0) *work = 0;
}

// FP32 constants of the pair loop, held in registers.
struct PairConst {
    float c2, n2, k3;
    float Lf[3], iLf[3];
};

// One slot pair (lane's i slot, j slot of this pass).  Masked-out slots take r^2 = rc^2, where the
// clamped switch polynomial is exactly 0, so every lane runs the same instructions.  The switch
// is f = A^2 B with A = rc^2 - u, B = 2u + rc^2 - 3 ron^2, u = r^2 clamped to [ron^2, rc^2]: the
// caller divides the sums by f(ron^2) (inv_f1), which makes inner pairs exactly 1.  Coulomb and
// LJ are summed as q_j g and eps_j l f; the row's q_i and eps_i multiply the sums at the end.
// WIDE: the cluster pair spans more than L - rc along an axis, so each displacement takes the
// minimum image.
template <bool NEWTON, bool WIDE>
__device__ __forceinline__ void cluster_pair(float dix, float diy, float diz, const float4& pj, const float4& qj,
                                             float si, bool in, const PairConst& K, float& pc, float& cl, float& vs) {
    float dx = dix + pj.x, dy = diy + pj.y, dz = diz + pj.z;
    if (WIDE) {
        dx = fmaf(-K.Lf[0], rintf(dx * K.iLf[0]), dx);
        dy = fmaf(-K.Lf[1], rintf(dy * K.iLf[1]), dy);
        dz = fmaf(-K.Lf[2], rintf(dz * K.iLf[2]), dz);
    }
    float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
    r2 = in ? r2 : K.c2;
    const float u = fminf(fmaxf(r2, K.n2), K.c2);
    const float a = K.c2 - u;
    const float f = a * a * fmaf(2.0f, u, K.k3);
    float rinv = rsqrtf(r2);
    if (NEWTON) rinv = rinv * fmaf(-0.5f * r2 * rinv, rinv, 1.5f);
    const float g = rinv * f;
    pc = fmaf(pj.w, g, pc);
    cl = fmaf(qj.x, g, cl);
    const float y = (si + qj.z) * rinv;
    const float x2 = y * y;
    const float x6 = x2 * x2 * x2;
    vs = fmaf(qj.y, fmaf(x6, x6, -x6) * f, vs);
}

// Distance test of cluster box (cA, hA) against half-cluster box (cB, hB) displaced by D: the
// boxes' gap is within the prune radius, or the pair is wide (spans L - rc along an axis, where
// another image of some atom pair may be the near one: never pruned).
__device__ __forceinline__ void box_test(float Dx, float Dy, float Dz, const float4& cA, const float4& hA,
                                         const float4& cB, const float4& hB, const ClusterGeom& G, bool& act,
                                         bool& wide) {
    const float gx = fabsf(Dx + cB.x - cA.x), gy = fabsf(Dy + cB.y - cA.y), gz = fabsf(Dz + cB.z - cA.z);
    const float sx = hA.x + hB.x, sy = hA.y + hB.y, sz = hA.z + hB.z;
    const float ex = fmaxf(gx - sx, 0.f), ey = fmaxf(gy - sy, 0.f), ez = fmaxf(gz - sz, 0.f);
    wide = gx + sx >= G.lim[0] || gy + sy >= G.lim[1] || gz + sz >= G.lim[2];
    act = wide || fmaf(ex, ex, fmaf(ey, ey, ez * ez)) <= G.prune2;
}

template <bool NEWTON, bool WIDE>
__device__ __forceinline__ void cluster_pair2(const float4& dd, const uint2& m2, const float4& pi, const float4& qi,
                                              const float4* __restrict__ sj, int jsub, unsigned lbit, const PairConst& K,
                                              float& ch, float& cl, float& vs) {
    const float dix = dd.x - pi.x, diy = dd.y - pi.y, diz = dd.z - pi.z;
    const float4 pj0 = sj[2 * jsub], qj0 = sj[2 * jsub + 1], pj1 = sj[2 * jsub + 8], qj1 = sj[2 * jsub + 9];
    float pc = 0.f;
    cluster_pair<NEWTON, WIDE>(dix, diy, diz, pj0, qj0, qi.z, (m2.x & lbit) != 0u, K, pc, cl, vs);
    cluster_pair<NEWTON, WIDE>(dix, diy, diz, pj1, qj1, qi.z, (m2.y & lbit) != 0u, K, pc, cl, vs);
    float sm, er;
    two_sum(ch, pc, sm, er);
    ch = sm;
    cl += er;
}

// Work distribution: each CTA takes 8 consecutive i-clusters at a time from a global counter
// (one per warp), so its warps work on neighbouring clusters and share their j-clusters in L1.
// Per warp, the 256 bytes of slot data of each j-cluster are staged in shared memory by one
// 8-byte load per lane, issued one cluster pair ahead.
template <bool NEWTON, int MINB>
__global__ void __launch_bounds__(256, MINB) k_energy_cluster(const uint4* __restrict__ cref, const float4* __restrict__ cctr,
                                                              const float4* __restrict__ chalf, const float4* __restrict__ hbox,
                                                              const float4* __restrict__ sdat, const int* __restrict__ cp_count,
                                                              const int4* __restrict__ cpl, int capP, int ncl, ClusterGeom G,
                                                              double* __restrict__ part, int* __restrict__ work) {
    __shared__ float4 s_d[8][32];
    __shared__ uint2 s_m[8][32];
    __shared__ __align__(16) float4 s_j[8][2][16];
    __shared__ int s_chunk[2];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const unsigned lbit = 1u << lane;
    const int islot = lane & 7, jsub = lane >> 3;
    const float2* __restrict__ sd2 = reinterpret_cast<const float2*>(sdat);
    PairConst K;
    K.c2 = G.c2; K.n2 = G.n2; K.k3 = G.k3;
#pragma unroll
    for (int k = 0; k < 3; k++) { K.Lf[k] = G.Lf[k]; K.iLf[k] = G.iLf[k]; }
    for (int it = 0;; it++) {
        if (threadIdx.x == 0) s_chunk[it & 1] = atomicAdd(work, 8);
        __syncthreads();
        const int A = s_chunk[it & 1] + w;
        if (s_chunk[it & 1] >= ncl) break;      // block-uniform
        if (A >= ncl) continue;
        const float4 pi = sdat[2 * (A * CL + islot)];       // (offset, q hi)
        const float4 qi = sdat[2 * (A * CL + islot) + 1];   // (q lo, eps, sig)
        const uint4 rA = cref[A];
        const float4 cA = cctr[A], hA = chalf[A];
        const int m = cp_count[A];
        const int4* row = cpl + (size_t)A * capP;
        float ch = 0.f, cl = 0.f;
        double vd = 0.0;
        for (int k0 = 0; k0 < m; k0 += 32) {
            float vs = 0.f;   // LJ of this batch of cluster pairs (at most 64 terms per lane)
            const int k = k0 + lane;
            bool act = false;
            float4 d = make_float4(0.f, 0.f, 0.f, 0.f);
            uint2 mm = make_uint2(0u, 0u);
            if (k < m) {
                // both halves of cluster B (slots 0-3, 4-7) are tested against A's box
                const int4 e = row[k];
                const uint4 rB = cref[e.x];
                const float4 cB0 = hbox[4 * e.x], hB0 = hbox[4 * e.x + 1], cB1 = hbox[4 * e.x + 2], hB1 = hbox[4 * e.x + 3];
                const float Dx = fixed_delta(rA.x, rB.x, G.Ls[0], G.Ll[0]);
                const float Dy = fixed_delta(rA.y, rB.y, G.Ls[1], G.Ll[1]);
                const float Dz = fixed_delta(rA.z, rB.z, G.Ls[2], G.Ll[2]);
                bool a0, a1, w0, w1;
                box_test(Dx, Dy, Dz, cA, hA, cB0, hB0, G, a0, w0);
                box_test(Dx, Dy, Dz, cA, hA, cB1, hB1, G, a1, w1);
                mm = make_uint2((unsigned)e.y, (unsigned)e.z);
                act = a0 || a1;
                d = make_float4(Dx, Dy, Dz, __int_as_float(e.x | ((w0 || w1) ? (int)0x80000000 : 0)));
            }
            const unsigned bal = __ballot_sync(0xffffffffu, act);
            if (act) {
                const int pos = __popc(bal & (lbit - 1u));
                s_d[w][pos] = d;
                s_m[w][pos] = mm;
            }
            __syncwarp();
            const int na = __popc(bal);
            float2 nx = make_float2(0.f, 0.f);
            if (na > 0) nx = sd2[(size_t)(__float_as_int(s_d[w][0].w) & 0x7fffffff) * 32 + lane];
            for (int t = 0; t < na; t++) {
                float2* sjw = reinterpret_cast<float2*>(s_j[w][t & 1]);
                sjw[lane] = nx;
                __syncwarp();
                if (t + 1 < na) nx = sd2[(size_t)(__float_as_int(s_d[w][t + 1].w) & 0x7fffffff) * 32 + lane];
                const float4 dd = s_d[w][t];
                const uint2 m2 = s_m[w][t];
                if (__float_as_int(dd.w) < 0)
                    cluster_pair2<NEWTON, true>(dd, m2, pi, qi, s_j[w][t & 1], jsub, lbit, K, ch, cl, vs);
                else
                    cluster_pair2<NEWTON, false>(dd, m2, pi, qi, s_j[w][t & 1], jsub, lbit, K, ch, cl, vs);
            }
            vd += (double)vs;
            __syncwarp();
        }
        // the lane's partial row: q_i (hi + lo) times the charge-weighted sum, eps_i times the LJ sum
        double e = ((double)pi.w + (double)qi.x) * ((double)ch + (double)cl);
        double v = (double)qi.y * vd;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            e += __shfl_xor_sync(0xffffffffu, e, o);
            v += __shfl_xor_sync(0xffffffffu, v, o);
        }
        if (lane == 0) {
            part[2 * A] = e * G.inv_f1;
            part[2 * A + 1] = v * G.inv_f1;
        }
    }
}

// ---- host ----------------------------------------------------------------------------------
template <typename T>
static int cl_alloc(T** p, size_t count) {
    if (*p) cudaFree(*p);
    *p = nullptr;
    cudaError_t e = cudaMalloc((void**)p, std::max<size_t>(count, 1) * sizeof(T));
    if (e != cudaSuccess) return fail(MCG_ECUDA, std::string("cudaMalloc: ") + cudaGetErrorString(e));
    return MCG_OK;
}

void ClusterPairs::release() {
    void* ptrs[] = {d_col_of, d_col_count, d_col_start, d_ccl_start, d_col_fill, d_col_atoms, d_cl_atom, d_cl_of, d_cref,
                    d_cctr, d_chalf, d_sdat, d_hbox, d_cp_count, d_cpl, d_misc, d_work};
    for (void* p : ptrs) if (p) cudaFree(p);
    d_col_of = d_col_count = d_col_start = d_ccl_start = d_col_fill = d_col_atoms = d_cl_atom = d_cl_of = nullptr;
    d_cref = nullptr; d_cctr = d_chalf = d_sdat = d_hbox = nullptr; d_cp_count = nullptr; d_cpl = nullptr;
    d_misc = nullptr; d_work = nullptr;
    ncol_cap = n_cap = ncl_cap = capP = 0;
    cpl_cap = 0;
    ok = false;
}

int ClusterPairs::build(cudaStream_t st, const uint4* fx, int n, const double L[3], const int* nbr, const int* nup,
                        const int* nlo, int cap) {
    ok = false;
    int rc;
    // columns of about one cluster's cross-section: edge = (8 V / n)^(1/3)
    const double vol = L[0] * L[1] * L[2];
    const double edge = std::cbrt(CL * vol / std::max(n, 1));
    ncx = std::max(1, (int)std::floor(L[0] / edge));
    ncy = std::max(1, (int)std::floor(L[1] / edge));
    while ((long long)ncx * ncy > (1 << 22)) { ncx = std::max(1, ncx / 2); ncy = std::max(1, ncy / 2); }
    ncol = ncx * ncy;
    if (ncol > ncol_cap) {
        if ((rc = cl_alloc(&d_col_count, ncol)) || (rc = cl_alloc(&d_col_start, ncol + 1)) ||
            (rc = cl_alloc(&d_ccl_start, ncol + 1)) || (rc = cl_alloc(&d_col_fill, ncol)))
            return rc;
        ncol_cap = ncol;
    }
    if (n > n_cap) {
        if ((rc = cl_alloc(&d_col_of, n)) || (rc = cl_alloc(&d_col_atoms, n)) || (rc = cl_alloc(&d_cl_of, n))) return rc;
        n_cap = n;
    }
    if (!d_misc) {
        if ((rc = cl_alloc(&d_misc, 8)) || (rc = cl_alloc(&d_work, 1))) return rc;
    }
    CKC(cudaMemsetAsync(d_col_count, 0, sizeof(int) * ncol, st));
    CKC(cudaMemsetAsync(d_misc, 0, sizeof(unsigned long long) * 8, st));
    k_col_assign<<<(n + 255) / 256, 256, 0, st>>>(fx, n, ncx, ncy, d_col_of, d_col_count);
    k_col_scan<<<1, 1024, 0, st>>>(d_col_count, ncol, d_col_start, d_ccl_start, d_col_fill, d_misc);
    k_col_scatter<<<(n + 255) / 256, 256, 0, st>>>(d_col_of, n, d_col_start, d_col_fill, d_col_atoms);
    CKC(cudaGetLastError());
    int tot_cl = 0;
    unsigned long long maxcol = 0;
    CKC(cudaMemcpyAsync(&tot_cl, d_ccl_start + ncol, sizeof(int), cudaMemcpyDeviceToHost, st));
    CKC(cudaMemcpyAsync(&maxcol, d_misc, sizeof(unsigned long long), cudaMemcpyDeviceToHost, st));
    CKC(cudaStreamSynchronize(st));
    build_launches += 3;
    if (maxcol > (unsigned long long)COL_SORT_MAX) return fail(MCG_ECAPACITY, "cluster build: a column holds too many atoms");
    ncl = tot_cl;
    const int nwords = (ncl + 31) / 32;
    if ((size_t)nwords * 8 + 8 * 64 > PAIR_SMEM_MAX) return fail(MCG_ECAPACITY, "cluster build: too many clusters");
    if (ncl > ncl_cap) {
        if ((rc = cl_alloc(&d_cl_atom, (size_t)ncl * CL)) || (rc = cl_alloc(&d_cref, ncl)) || (rc = cl_alloc(&d_cctr, ncl)) ||
            (rc = cl_alloc(&d_chalf, ncl)) || (rc = cl_alloc(&d_sdat, (size_t)ncl * CL * 2)) || (rc = cl_alloc(&d_cp_count, ncl)) ||
            (rc = cl_alloc(&d_hbox, (size_t)ncl * 4)))
            return rc;
        ncl_cap = ncl;
        capP = 0;
    }
    int m2 = 1;
    while ((unsigned long long)m2 < maxcol) m2 <<= 1;
    const size_t sort_smem = (size_t)m2 * sizeof(unsigned long long);
    CKC(cudaFuncSetAttribute(k_col_sort, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)std::max<size_t>(sort_smem, 1024)));
    k_col_sort<<<ncol, 256, sort_smem, st>>>(fx, d_col_start, d_ccl_start, d_col_atoms, d_cl_atom, d_cl_of);
    CKC(cudaGetLastError());
    build_launches += 1;
    if (capP == 0) capP = 256;
    for (int attempt = 0; attempt < 3; attempt++) {
        const size_t smem = (size_t)nwords * 8 + (size_t)capP * 8;
        if (smem > PAIR_SMEM_MAX) return fail(MCG_ECAPACITY, "cluster build: pair-list row too long");
        if ((size_t)ncl * capP > cpl_cap) {
            if ((rc = cl_alloc(&d_cpl, (size_t)ncl * capP))) return rc;
            cpl_cap = (size_t)ncl * capP;
        }
        CKC(cudaMemsetAsync(d_misc + 1, 0, sizeof(unsigned long long) * 3, st));
        CKC(cudaFuncSetAttribute(k_cluster_pairs, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        k_cluster_pairs<<<ncl, 256, smem, st>>>(d_cl_atom, d_cl_of, nbr, nup, nlo, cap, nwords, capP, d_cp_count, d_cpl, d_misc);
        CKC(cudaGetLastError());
        build_launches += 1;
        unsigned long long mres[3] = {0, 0, 0};
        CKC(cudaMemcpyAsync(mres, d_misc + 1, sizeof(mres), cudaMemcpyDeviceToHost, st));
        CKC(cudaStreamSynchronize(st));
        if (mres[0] == 0) {
            nbits = (int64_t)mres[1];
            npairs = (int64_t)mres[2];
            ok = true;
            return MCG_OK;
        }
        capP = (int)((mres[0] * 5 / 4 + 31) & ~31ull);
    }
    return fail(MCG_ECAPACITY, "cluster build: pair-list capacity could not be grown");
}

int ClusterPairs::launch_energy(cudaStream_t st, int v, const uint4* fx, const float4* prmf, const ClusterGeom& G,
                                double* part) {
    const int nslot = ncl * CL;
    k_cluster_pack<<<(nslot + 255) / 256, 256, 0, st>>>(fx, prmf, d_cl_atom, ncl, G, d_cref, d_cctr, d_chalf, d_sdat,
                                                       d_hbox, d_work);
    // the reciprocal square root takes one Newton step (the bare hardware estimate biases the
    // Coulomb sum by ~2e-7 relative); variants differ in resident CTAs per SM
    switch (v) {
    case 0:
        k_energy_cluster<true, 3><<<152 * 3, 256, 0, st>>>(d_cref, d_cctr, d_chalf, d_hbox, d_sdat, d_cp_count, d_cpl, capP,
                                                          ncl, G, part, d_work);
        break;
    default:
        k_energy_cluster<true, 4><<<152 * 4, 256, 0, st>>>(d_cref, d_cctr, d_chalf, d_hbox, d_sdat, d_cp_count, d_cpl, capP,
                                                          ncl, G, part, d_work);
        break;
    }
    return ncl;
}

}  // namespace mcg
