// Batched independent NVT chains: one persistent CTA per chain per sweep.
//
// Each chain is a box of identical rigid residues (1..8 atoms: argon, 3-site water ...).  A sweep
// is nres trial moves per chain, performed in order as MC_metropolis::run does
// (src/MC_metropolis.cpp:80-165): pick TRN or ROT uniformly, a residue uniformly and, for ROT, a
// pivot atom of it uniformly (the reference lists one move instance per selected atom,
// List_Moves.cpp:393-440), draw a displacement uniform in the dmax ball or an axis and an angle
// uniform in [-dmax, dmax] degrees, compute dE against the residue's neighbours, accept with the
// Metropolis test (MC_metropolis.cpp:175-204).  Differences from the reference, all deliberate:
// random numbers come from a per-chain Philox4x32-10 stream (counter = move index), rotations use
// the minimum-image offset from the pivot (the reference rotates raw coordinates of residues
// straddling the box, Move.hpp:145-183, and can tear them apart), and the neighbour list is
// rebuilt whenever an atom has moved more than half the skin since the last build (the reference
// rebuilds every 50 steps whatever the displacement, MC_metropolis.cpp:151), so no pair inside
// the cutoff is ever missed.
//
// HBM layout (pools over all chains, chain c owns a contiguous slice):
//   M[atoms]      ulonglong4_32a  master coordinates as 64-bit fixed-point box fractions (x, y, z):
//                 exact, wrap-free integer updates, resolution L/2^64 (finer than FP64 anywhere in
//                 the box); FP64 views (x = int64 * L/2^64) are formed only for output and checks
//   F[atoms]      uint4    32-bit mirror = the high words of M (w = residue slot type)
//   FB[atoms]     uint4    mirror positions at the last list build (displacement check)
//   LST[res*cap]  uint16   neighbour residues of each residue (any atom pair within rc + skin)
//   NL[res]       int      list lengths
//   chains[c]     ChainDev parameters; state[c] ChainState counters and the running energy
//
// Precision: 64-bit fixed-point master coordinates (the box wrap is the integer overflow), FP64
// running energy, dE sum and acceptance threshold -ln(alpha)/beta; FP32 pair terms on exact
// fixed-point displacements (mixed_pair_delta).  GB300's FP64 rate is a small fraction of its
// FP32 rate, so no FP64 arithmetic sits on the per-move critical path except one compare: the
// threshold is computed by a warp that would otherwise wait at the barrier.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <map>
#include <mutex>
#include <numeric>
#include <string>
#include <vector>

#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include "engine.hpp"
#include "mcg.h"
#include "pair_math.cuh"

namespace mcg {

#define BK(call)                                                                              \
    do {                                                                                      \
        cudaError_t e_ = (call);                                                              \
        if (e_ != cudaSuccess) return fail(MCG_ECUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

constexpr int MAX_APR = 8;
constexpr int MAX_CELLS = 4096;
constexpr double TWO64 = 18446744073709551616.0;

// ---- Philox4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as easy as 1, 2, 3",
// SC'11): 10 rounds of the 4x32 Philox S-box with the published multipliers and Weyl key
// increments.
struct U4 { uint32_t x, y, z, w; };

__device__ __forceinline__ U4 philox4x32_10(U4 ctr, uint32_t k0, uint32_t k1) {
    const uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u, W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
#pragma unroll
    for (int r = 0; r < 10; r++) {
        uint32_t hi0 = __umulhi(M0, ctr.x), lo0 = M0 * ctr.x;
        uint32_t hi1 = __umulhi(M1, ctr.z), lo1 = M1 * ctr.z;
        ctr = U4{hi1 ^ ctr.y ^ k0, lo1, hi0 ^ ctr.w ^ k1, lo0};
        k0 += W0;
        k1 += W1;
    }
    return ctr;
}

__device__ __forceinline__ float u01f(uint32_t v) { return (float)(v >> 8) * (1.0f / 16777216.0f); }
// (0, 1]: never 0, so -ln(alpha) is finite
__device__ __forceinline__ double u01d_open0(uint32_t hi, uint32_t lo) {
    return ((double)(((uint64_t)hi << 21) ^ (uint64_t)(lo >> 11)) + 1.0) * (1.0 / 9007199254740992.0);
}

struct ChainDev {
    int atom0, res0, nres, apr;
    double L[3], rL[3];
    float tofix32[3];     // 2^32 / L : Angstrom -> mirror units (master increments, master_step)
    int nc[3];            // cell grid for list builds
    int use_cells;        // 0: boxes too small for a 5-cell stencil; every residue is scanned
    int kspec;            // moves evaluated together by the sweep (1, 2, 4, 8, 16 or 32)
    int wrap_offsets;     // box small enough that (b - a_0) - (a_k - a_0) may leave the minimum image
    float Lf[3], Lhalf[3];
    float Ls[3], Lsl[3];  // L / 2^32 as float-float: mirror units -> Angstrom
    double beta;
    float beta_f;         // beta rounded to FP32 (clear-margin Metropolis decisions)
    float dmax_trn, dmax_rot;
    int ntypes_move;      // 1: TRN only, 2: TRN + ROT
    int each[2];          // dmax adjustment period per move type (0 = fixed), MC::adjust_dmax
    double target[2];     // target acceptance per move type, fraction
    double dmax_cap[2];   // largest adjusted dmax per move type
    uint32_t key0, key1;
    float tab[MAX_APR][MAX_APR][4];   // (qk, e4, ss, qk_lo) per slot pair; qk + qk_lo = K q_a q_b
    float tablo[MAX_APR][MAX_APR][2]; // (e4_lo, ss_lo): float-float parts for total-energy kernels
};

struct ChainState {
    double etot;
    long long trials, accepted;
    long long pairs;            // pair interactions evaluated (inside rc before or after a move)
    unsigned long long moves;   // Philox counter
    int rebuilds;               // list builds (before or during sweeps)
    int err;
    float maxd2;                // largest squared displacement of a committed atom since the last build
    int pad_;
    double dmax[2];             // current dmax: translation (A), rotation (degrees)
    int acc_tmp[2];             // accepted moves per type since the last dmax adjustment
};

struct BatchGeom {
    float c2f, n2f, sw2f;
    float rlist2;      // (rc + skin)^2
    float rcent2;      // (rc + skin + 2 rext)^2, residue-centre prefilter
    float half_skin2;  // (skin/2)^2
    float cellmin;     // cell edge for the 5-stencil
    float indep2;      // (rc + 2 extents + 2 largest moves)^2: two moves cannot interact beyond it
    float subst2;      // (list centre radius + skin)^2: a residue farther than this is in no list of the other
    float pre2;        // a chain whose atoms moved less than this (squared) since the build keeps its lists
    float pair2;       // (rc + 2 extents)^2: residues whose first atoms are farther share no atom pair within rc
    int cap;
};

__device__ __forceinline__ float fdelta(uint32_t a, uint32_t b, float Lh, float Ll) { return fixed_delta(a, b, Lh, Ll); }

__device__ __forceinline__ int cell_coord(uint32_t v, int nc) {
    return (int)((((v + 0x80000000u) >> 8) * (uint64_t)nc) >> 24);
}

// ---- neighbour lists ----------------------------------------------------------------------
// Residues are binned by their first atom into cells of edge >= (rc + skin + 2 rext)/2 and a
// 5x5x5 stencil is scanned; boxes with fewer than 5 cells per edge scan every residue.  A residue
// q enters the list of r when their first atoms are within rc + skin + 2 extents (a superset of the
// residues with an atom pair within rc + skin).  Before a sweep, a grid-wide pass (k_batch_bin +
// k_batch_lists) rebuilds the lists of the chains whose atoms have moved more than 0.7 half-skins
// since their last build; inside a sweep, a chain whose atom has moved more than half the skin
// rebuilds its own lists with its CTA (chain_rebuild) before the next move.  Lists are built a home
// cell per warp: lane = home residue, candidates staged 32 at a time in shared memory.

// Block-level binning of chain C: copies the build positions and, when the chain uses cells,
// fills starts[0..ncell] (shared or global) and g_order (residues sorted by cell, then index).
__device__ void chain_bin(const ChainDev& C, const uint4* __restrict__ F, uint4* FB, int* starts, int* g_order,
                          int* g_cell, uint4* g_pos) {
    const int apr = C.apr, nres = C.nres;
    const int T = blockDim.x, tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nw = T >> 5;
    const uint4* Fc = F + C.atom0;
    for (int i = tid; i < nres * apr; i += T) FB[C.atom0 + i] = Fc[i];
    if (!C.use_cells) { __syncthreads(); return; }
    const int ncell = C.nc[0] * C.nc[1] * C.nc[2];
    for (int c = tid; c <= ncell; c += T) starts[c] = 0;
    __syncthreads();
    for (int r = tid; r < nres; r += T) {
        const uint4 p = Fc[r * apr];
        const int c = (cell_coord(p.z, C.nc[2]) * C.nc[1] + cell_coord(p.y, C.nc[1])) * C.nc[0] + cell_coord(p.x, C.nc[0]);
        g_cell[r] = c;
        atomicAdd(&starts[c + 1], 1);
    }
    __syncthreads();
    if (tid == 0)
        for (int c = 1; c <= ncell; c++) starts[c] += starts[c - 1];
    __syncthreads();
    // starts[c] doubles as the fill cursor of cell c; restored afterwards
    for (int r = tid; r < nres; r += T) g_order[atomicAdd(&starts[g_cell[r]], 1)] = r;
    __syncthreads();
    if (tid == 0) {
        for (int c = ncell; c >= 1; c--) starts[c] = starts[c - 1];
        starts[0] = 0;
    }
    __syncthreads();
    // sort each cell so the list order (and the dE summation order) is deterministic
    for (int c = warp; c < ncell; c += nw) {
        const int b = starts[c], e = starts[c + 1], m = e - b;
        if (m <= 1) continue;
        if (m <= 32) {
            int v = lane < m ? g_order[b + lane] : 0x7fffffff;
            for (int k = 2; k <= 32; k <<= 1)
                for (int j = k >> 1; j > 0; j >>= 1) {
                    const int o = __shfl_xor_sync(0xffffffffu, v, j);
                    const bool up = (lane & k) == 0, lower = (lane & j) == 0;
                    v = (lower == up) ? min(v, o) : max(v, o);
                }
            if (lane < m) g_order[b + lane] = v;
        } else if (lane == 0) {
            for (int i = b + 1; i < e; i++) {
                int v = g_order[i], k = i - 1;
                while (k >= b && g_order[k] > v) { g_order[k + 1] = g_order[k]; k--; }
                g_order[k + 1] = v;
            }
        }
    }
    __syncthreads();
    // first-atom positions in cell order: the candidate scan reads them contiguously
    for (int t = tid; t < nres; t += T) {
        uint4 p = Fc[g_order[t] * apr];
        p.w = (uint32_t)g_order[t];
        g_pos[t] = p;
    }
    __syncthreads();
}

// The contiguous slot ranges of the 5x5x5 stencil around home cell (hx, hy, hz), in stencil
// order: the 25 (dz, dy) rows, each the merged ranges of its five x cells in dx order.
template <typename Fn>
__device__ __forceinline__ void stencil_ranges(const ChainDev& C, const int* __restrict__ starts, int hx, int hy, int hz,
                                               Fn&& f) {
    const int nx = C.nc[0], ny = C.nc[1], nz = C.nc[2];
    for (int dz = -2; dz <= 2; dz++) {
        int z = hz + dz;
        z += z < 0 ? nz : (z >= nz ? -nz : 0);
        for (int dy = -2; dy <= 2; dy++) {
            int y = hy + dy;
            y += y < 0 ? ny : (y >= ny ? -ny : 0);
            const int rowc = (z * ny + y) * nx;
            int rb = -1, re = -1;
            for (int dx = -2; dx <= 2; dx++) {
                int x = hx + dx;
                x += x < 0 ? nx : (x >= nx ? -nx : 0);
                const int b = starts[rowc + x], e = starts[rowc + x + 1];
                if (b == re) { re = e; continue; }
                if (re > rb) f(rb, re);
                rb = b;
                re = e;
            }
            if (re > rb) f(rb, re);
        }
    }
}

// Lists of the residues of one work item of chain C (all 32 lanes of the calling warp): a home
// cell when the chain uses cells, else 32 consecutive residues scanning every residue.  Lanes take
// the candidates 32 at a time (the stencil's merged cell rows, at most two per (dz, dy) row of the
// stencil); each chunk is tested against the home residues in turn (positions read from shared
// memory; lane h holds home residue h's row count), and the candidates within range are appended
// to that residue's row by a ballot, in candidate order.  `stage`: a per-warp shared-memory buffer
// of 64 uint4, the ranges in its first half and the home residues in its second.
template <int APR>
__device__ void item_lists(const ChainDev& C, const BatchGeom& G, const uint4* __restrict__ Fc, int item,
                           const int* __restrict__ starts, const int* __restrict__ g_order,
                           const uint4* __restrict__ g_pos, uint16_t* LST, int* NL, int* err_out, uint4* stage) {
    (void)g_order;
    const int apr = APR ? APR : C.apr;
    const int lane = threadIdx.x & 31;
    const unsigned lt_mask = (1u << lane) - 1u;
    const bool cells = C.use_cells != 0;
    const float Lf0 = C.Ls[0] + C.Lsl[0], Lf1 = C.Ls[1] + C.Lsl[1], Lf2 = C.Ls[2] + C.Lsl[2];
    const float rc2 = G.rcent2;
    const int cap = G.cap;
    int hb, he;
    int2* rng = reinterpret_cast<int2*>(stage);      // up to 50 ranges (400 bytes)
    uint4* home = stage + 32;                          // the home residues of the current pass
    int nr = 0;
    if (cells) {
        hb = starts[item];
        he = starts[item + 1];
        const int hx = item % C.nc[0], hy = (item / C.nc[0]) % C.nc[1], hz = item / (C.nc[0] * C.nc[1]);
        stencil_ranges(C, starts, hx, hy, hz, [&](int b, int e) {
            if (lane == 0) rng[nr] = make_int2(b, e);
            nr++;
        });
    } else {
        hb = item * 32;
        he = min(C.nres, hb + 32);
        if (lane == 0) rng[0] = make_int2(0, C.nres);
        nr = 1;
    }
    __syncwarp();
    for (int h0 = hb; h0 < he; h0 += 32) {
        // up to 32 home residues at a time: lane h holds home residue h0 + h, its position and its
        // row's entry count
        const int nh = min(32, he - h0);
        uint4 ph = make_uint4(0, 0, 0, 0);
        int rh = 0;
        if (lane < nh) {
            if (cells) { ph = g_pos[h0 + lane]; rh = (int)ph.w; }
            else { rh = h0 + lane; ph = Fc[(size_t)rh * apr]; }
            ph.w = (uint32_t)rh;
            home[lane] = ph;
        }
        __syncwarp();
        int cnt = 0;
        for (int q = 0; q < nr; q++) {
            const int2 be = rng[q];
            for (int k = be.x; k < be.y; k += 32) {
                const int t = k + lane;
                const bool valid = t < be.y;
                uint4 v = make_uint4(0, 0, 0, 0);
                if (valid) {
                    if (cells) v = g_pos[t];            // w = residue index
                    else { v = Fc[(size_t)t * apr]; v.w = (uint32_t)t; }
                }
                for (int h = 0; h < nh; h++) {
                    const uint4 hp = home[h];           // broadcast: position and residue index of home h
                    const int r = (int)hp.w;
                    // displacements with the FP32 scale L / 2^32 (rounded): the list radius carries a
                    // 0.01 A margin, far above the ~1e-6 A this rounding moves a distance
                    const float dx = __int2float_rn((int)(v.x - hp.x)) * Lf0, dy = __int2float_rn((int)(v.y - hp.y)) * Lf1,
                                dz = __int2float_rn((int)(v.z - hp.z)) * Lf2;
                    const bool keep = valid && (int)v.w != r && dx * dx + dy * dy + dz * dz <= rc2;
                    const unsigned bal = __ballot_sync(0xffffffffu, keep);
                    const int pos = __shfl_sync(0xffffffffu, cnt, h) + __popc(bal & lt_mask);
                    if (keep && pos < cap) LST[(size_t)(C.res0 + r) * cap + pos] = (uint16_t)v.w;
                    if (lane == h) cnt += __popc(bal);
                }
            }
        }
        if (lane < nh) {
            NL[C.res0 + rh] = min(cnt, cap);
            if (cnt > cap) atomicExch(err_out, MCG_ECAPACITY);
        }
        __syncwarp();   // home[] is rewritten for the next home residues
    }
    __syncwarp();   // the range buffer is free for the warp's next item
}

__device__ __forceinline__ int chain_items(const ChainDev& C) {
    return C.use_cells ? C.nc[0] * C.nc[1] * C.nc[2] : (C.nres + 31) / 32;
}

// Per-chain binning before a sweep, one CTA of 1024 threads per chain: only chains that were asked
// to (force) or whose atoms moved more than sqrt(pre2) since their last build; build[c] tells
// k_batch_lists.
__global__ void __launch_bounds__(1024) k_batch_bin(const ChainDev* __restrict__ chains, const uint4* __restrict__ F, uint4* FB,
                                                    int* g_starts,
                            int* g_order, int* g_cell, uint4* g_pos, ChainState* state, int* build, float pre2, int force,
                            int nchains) {
    const int c = blockIdx.x;
    if (c >= nchains) return;
    const bool need = force || state[c].maxd2 > pre2;
    if (threadIdx.x == 0) build[c] = need ? 1 : 0;
    if (!need) return;
    const ChainDev& C = chains[c];
    // the cell starts are counted, summed and used as fill cursors in shared memory, then copied
    // out for k_batch_lists
    __shared__ int s_starts[MAX_CELLS + 1];
    chain_bin(C, F, FB, s_starts, g_order + C.res0, g_cell + C.res0, g_pos + C.res0);
    if (C.use_cells) {
        int* gs = g_starts + (size_t)c * (MAX_CELLS + 1);
        const int ncell = C.nc[0] * C.nc[1] * C.nc[2];
        for (int k = threadIdx.x; k <= ncell; k += blockDim.x) gs[k] = s_starts[k];
    }
    if (threadIdx.x == 0) {
        state[c].maxd2 = 0.0f;
        state[c].rebuilds++;
    }
}

// Lists of the chains binned by k_batch_bin: one warp per work item (home cell) over the GPU.
template <int APR>
__global__ void __launch_bounds__(256) k_batch_lists(const ChainDev* __restrict__ chains, BatchGeom G,
                                                     const uint4* __restrict__ F, const int* __restrict__ item_chain,
                                                     const int* __restrict__ chain_item0, const int* __restrict__ g_starts,
                                                     const int* __restrict__ g_order, const uint4* __restrict__ g_pos,
                                                     uint16_t* LST, int* NL, ChainState* state,
                                                     const int* __restrict__ build, int nitems) {
    __shared__ uint4 s_stage[8][64];   // per warp: the stencil's cell ranges and the home residues
    const int warp = threadIdx.x >> 5;
    const int warps = gridDim.x * 8;
    for (int it = blockIdx.x * 8 + warp; it < nitems; it += warps) {
        const int c = item_chain[it];
        if (!build[c]) continue;
        const ChainDev& C = chains[c];
        if (APR && C.apr != APR) continue;
        item_lists<APR>(C, G, F + C.atom0, it - chain_item0[c], g_starts + (size_t)c * (MAX_CELLS + 1), g_order + C.res0,
                        g_pos + C.res0, LST, NL, &state[c].err, s_stage[warp]);
    }
}

// In-sweep rebuild of one chain by its own CTA (shared-memory cell starts; `stage`: 32 entries
// per warp).
template <int APR>
__device__ void chain_rebuild(const ChainDev& C, const BatchGeom& G, const uint4* __restrict__ F, uint4* FB,
                              uint16_t* LST, int* NL, int* s_starts, int* g_order, int* g_cell, uint4* g_pos,
                              int* err_out, uint4* stage) {
    chain_bin(C, F, FB, s_starts, g_order, g_cell, g_pos);
    const int warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const int nitems = chain_items(C);
    for (int it = warp; it < nitems; it += nw)
        item_lists<APR>(C, G, F + C.atom0, it, s_starts, g_order, g_pos, LST, NL, err_out, stage);
    __syncthreads();
}

// ---- the sweep ------------------------------------------------------------------------------
constexpr int KMAX = 32;                 // moves evaluated together, at most (8 for residues of more than 4 atoms)
constexpr int RING = 64;                 // per-warp ring of compacted neighbour atoms (power of two)

// What every warp needs of a move after the iteration's barrier (written by the first warp of the
// move's group): residue, old and new positions of its atoms (interaction test, dE corrections,
// commit substitutes), build positions (far check) and the Metropolis draw.
// A: atoms per residue the kernel is compiled for (the record is sized for them).
template <int A>
struct MoveRec {
    uint4 fn[A];                         // new mirror positions (w = slot)
    uint4 fo[A];                         // old mirror positions
    unsigned long long mn[A][3];         // new master coordinates
    uint4 fb[A];                         // build positions of the moved atoms
    uint4 fo0;                           // old position of the first atom
    int res;
    int rot;                             // move type: 0 translation, 1 rotation
    float lna;                           // -ln(alpha), FP32 estimate (NaN: decide in FP64)
    uint32_t ahi, alo;                   // Philox words of alpha in (0, 1] (u01d_open0)
};

// Metropolis test (MC_metropolis.cpp:175-204): accept when dE <= DBL_EPSILON, else when
// alpha < exp(-beta dE).  dE = deh + del (float-float, iu).  Decided in FP32 when the margin is
// clear (FP32 dE and beta are within 1e-6 relative, lna within 2e-5), in FP64 otherwise.
template <int A>
__device__ __forceinline__ bool metropolis_accept(float deh, float del, const MoveRec<A>& Q, float beta_f, double beta) {
    const float hf = deh + del;
    if (hf <= 0.0f) return true;
    if (hf >= 1e-12f) {
        const float tf = beta_f * hf, lna = Q.lna;
        if (tf < lna - 1e-4f * fmaxf(1.0f, lna)) return true;
        if (tf > lna + 1e-4f * fmaxf(1.0f, lna)) return false;
        // inside the margin, or lna is NaN: FP64
    }
    const double de = (double)deh + (double)del;
    return de <= 2.220446049250313e-16 || u01d_open0(Q.ahi, Q.alo) < exp(-beta * de);
}

// This lane's share of the change in move g's dE when the earlier move h of the same iteration is
// accepted: the pair terms between the two residues, as differences between g's new and old
// positions, with h at its new positions minus with h at its old ones.  The 2 apr^2 atom-pair terms
// are spread over the warp's lanes; a pair out of range in both positions of g contributes exactly 0.
// The displacements come straight from the fixed-point mirrors (exact minimum images); g's new
// displacement is the old one less g's atom move, the minimum image for every pair within rc since
// rc + the largest move <= L/2.
template <int A, bool PK>
__device__ __forceinline__ float pair_correction(const MoveRec<A>& Qg, const MoveRec<A>& Qh, int apr, int lane,
                                                 const float4 (*tab)[MAX_APR], float Ls0, float Ls1, float Ls2,
                                                 float Ll0, float Ll1, float Ll2, float c2, float n2, float k3) {
    float s = 0.0f;
    const int npr = apr * apr;
    for (int t = lane; t < 2 * npr; t += 32) {
        const int side = t >= npr ? 1 : 0;                 // 0: h new (+), 1: h old (-)
        const int r = t - side * npr, j = r / apr, b = r - j * apr;
        const uint4 a = Qg.fo[j], an = Qg.fn[j];
        const uint4 hb = side ? Qh.fo[b] : Qh.fn[b];
        const float dx = fdelta(a.x, hb.x, Ls0, Ll0), dy = fdelta(a.y, hb.y, Ls1, Ll1), dz = fdelta(a.z, hb.z, Ls2, Ll2);
        const float mx = fdelta(a.x, an.x, Ls0, Ll0), my = fdelta(a.y, an.y, Ls1, Ll1), mz = fdelta(a.z, an.z, Ls2, Ll2);
        const float4 tb = tab[j][hb.w];
        int np = 0;
        const float v = pair_delta<PK>(dx, dy, dz, mx, my, mz, tb.x, tb.y, tb.z, c2, n2, k3, np);
        s += side ? -v : v;
    }
    return s;
}

// Per-move record of a logged sweep (mcg_batch_sweep_logged): the layout of mcg_batch_move, with
// the proposed positions as raw 64-bit masters (the host converts them to Angstrom in place).
struct MoveLogDev {
    double de;
    int res;
    int flags;                           // bit 0 rotation, bit 1 accepted
    uint32_t ahi, alo;
    unsigned long long pos[MAX_APR][3];
};
static_assert(sizeof(MoveLogDev) == sizeof(mcg_batch_move), "record layout of mcg_batch_move");

// Master-unit increment for a displacement d (Angstrom): d * 2^64 / L as a 64-bit integer, formed
// in FP32 + integer arithmetic (v = d * 2^32 / L; integer part -> high word, fraction -> low word).
__device__ __forceinline__ unsigned long long master_step(float d, float tofix32) {
    const float v = d * tofix32;
    const float fl = floorf(v);
    const int hi = __float2int_rn(fl);
    const uint32_t lo = __float2uint_rn((v - fl) * 4294967296.0f);   // (v - fl) < 1 exactly
    return ((unsigned long long)(long long)hi << 32) + lo;
}

// Speculative exact sweep.  Each iteration takes the next K moves of the chain (K = 1, 2, 4, 8, 16
// or 32 per chain); the NT/K threads of group g (whole warps) evaluate move mv+g against the state
// before the iteration.  After the iteration barrier the CTA tests every pair of moves (g, h < g)
// for a shared residue or possible interaction (first atoms within rc + 2 extents + 2 largest
// moves) and computes, for each interacting pair, the change of the pair terms between the two
// residues that h's move makes (h's new minus h's old positions); after a second, CTA-local
// barrier every warp decides the moves in order with the same data: g's dE is corrected by the
// terms of the earlier ACCEPTED moves that interact with it, so it is the dE the sequential chain
// computes, and the test is taken on it: the chain equals the sequential Metropolis chain up to
// FP32 summation order.  A move whose residue an earlier accepted move of the iteration moved, and
// all later ones, are re-proposed next iteration from the same Philox counters.
//
// Per iteration and warp: the warp draws its group's move from the Philox stream and applies it to
// its residue (lanes = atoms; every warp of a group does this redundantly, so no barrier is needed
// before the pair loop).  It then scans its share of the residue's neighbour list: the neighbour
// atoms whose distance from the residue's centroid is within rc + the residue's extent about the
// centroid + this move's largest atom displacement are compacted, as displacements from the first
// atom, into the warp's ring in shared memory, and each time 32 are pending they are evaluated
// with all lanes busy (old and new pair terms, mixed_pair_delta).  Commits are written by the
// first warp of each group
// after the barrier; positions that a warp may read before they land come from the previous
// iteration's move records instead.
//
// CL = 2: the chain runs on a cluster of two CTAs (two SMs).  Its K moves per iteration are split
// K/2 per CTA; each warp writes its partial dE and each group its move record to both CTAs'
// shared memory (distributed shared memory), and the iteration's barrier is the cluster barrier.
// In-sweep list rebuilds are done by CTA 0 while CTA 1 waits at the cluster barrier.
template <int APR, int NT, int CL>
__global__ void __launch_bounds__(NT, NT >= 512 ? 1 : (NT >= 256 ? 2 : (APR == 1 ? 8 : 4))) k_batch_sweep(const ChainDev* __restrict__ chains, BatchGeom G, ulonglong4_32a* M,
                                                       uint4* F, uint4* FB, uint16_t* LST, int* NL, int* g_order,
                                                       int* g_cell, uint4* g_pos, ChainState* state,
                                                       const int* __restrict__ cta_start,
                                                       const int* __restrict__ cta_chains, int nchains,
                                                       MoveLogDev* mlog) {
    namespace cg = cooperative_groups;
    constexpr int NW = NT / 32;
    constexpr int A = APR ? APR : MAX_APR;        // register arrays per moved atom
    // the pair delta on packed FP32, except in the one-atom 128-thread kernel held to 64 registers
    // (8 CTAs per SM), where the packed form's extra live registers spill
    constexpr bool PK = !(APR == 1 && NT == 128);
    static_assert(CL == 1 || CL == 2, "clusters of one or two CTAs");
    // moves per iteration, at most (shared-memory records): a warp per move at the least
    constexpr int KM = (A <= 4 ? KMAX : 8) < NT * CL / 32 ? (A <= 4 ? KMAX : 8) : NT * CL / 32;
    // The move records and the cell starts of an in-sweep list rebuild share their memory: a
    // rebuild runs after the iteration's decisions and commits, and the iteration after it reads
    // no record of the one before (its commits have landed).
    union SweepShared {
        MoveRec<A> P[2][KM];
        int cell[MAX_CELLS + 1];
    };
    __shared__ SweepShared s_u;
    auto& P = s_u.P;
    int* s_cell = s_u.cell;
    __shared__ float2 s_red[2][CL * NW];
    // per move: earlier moves of the iteration that may interact with it / moved its residue; two
    // buffers by iteration parity (an iteration clears its buffer before its first barrier)
    __shared__ unsigned s_cm[2][KM], s_sr[2][KM];
    __shared__ float2 s_corr[KM][KM];             // [g][h]: dE correction of move g if move h is accepted
    __shared__ float4 s_ring[NW][RING];
    __shared__ int s_err;
    __shared__ float4 s_tab[MAX_APR][MAX_APR];        // 16-byte aligned: read as float4
    __shared__ unsigned long long s_pairs;
    __shared__ __align__(16) ChainDev s_chain;        // the chain's constants, off the global-memory path
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const unsigned lt_mask = (1u << lane) - 1u;
    float4* ring = s_ring[warp];
    const int rank = CL > 1 ? (int)cg::this_cluster().block_rank() : 0;
    const int unit = blockIdx.x / CL;                 // the CTA (or cluster) in the chain packing
    // the iteration barrier: the CTA, or both CTAs of the cluster (memory visible across them)
    auto unit_sync = [&]() {
        if (CL > 1) cg::this_cluster().sync();
        else __syncthreads();
    };
    // the other CTA's copy of a shared-memory object (CL = 2)
    auto peer = [&](auto* p) { return CL > 1 ? cg::this_cluster().map_shared_rank(p, rank ^ 1) : p; };
    for (int slot = cta_start[unit]; slot < cta_start[unit + 1]; slot++) {
        const int c = cta_chains[slot];
        if (c >= nchains) continue;
        if (APR && chains[c].apr != APR) continue;
        unit_sync();   // the previous chain's last reads of shared state are done (in both CTAs)
        {
            static_assert(sizeof(ChainDev) % 4 == 0, "ChainDev copied as words");
            const int* src = reinterpret_cast<const int*>(&chains[c]);
            int* dst = reinterpret_cast<int*>(&s_chain);
            for (int k = tid; k < (int)(sizeof(ChainDev) / 4); k += NT) dst[k] = src[k];
        }
        __syncthreads();
        const ChainDev& C = s_chain;
        const int apr = APR ? APR : C.apr;
        const int K = C.kspec;                 // 1, 2, 4, 8, 16 or 32 (<= KM); CL * NT / K >= 32
        const int KL = K / CL;                 // moves of this CTA
        const int GS = NT / KL;                // threads per move
        const int WPG = GS >> 5;               // warps per move
        const int grp = rank * KL + tid / GS, gw = ((tid % GS) >> 5);
        const float Ls0 = C.Ls[0], Ls1 = C.Ls[1], Ls2 = C.Ls[2], Ll0 = C.Lsl[0], Ll1 = C.Lsl[1], Ll2 = C.Lsl[2];
        // (qk sw2, e4 sw2, ss, qk_lo): the switch normalisation folded into the pair constants
        for (int k = tid; k < MAX_APR * MAX_APR; k += NT)
            s_tab[k / MAX_APR][k % MAX_APR] = make_float4(
                (float)((double)C.tab[k / MAX_APR][k % MAX_APR][0] * (double)G.sw2f),
                (float)((double)C.tab[k / MAX_APR][k % MAX_APR][1] * (double)G.sw2f), C.tab[k / MAX_APR][k % MAX_APR][2],
                C.tab[k / MAX_APR][k % MAX_APR][3]);
        const float c2f = G.c2f, n2f = G.n2f, k3f = G.c2f - 3.0f * G.n2f, rcf = sqrtf(G.c2f);
        ChainState S = state[c];
        if (tid == 0) { s_err = 0; s_pairs = 0ull; }
        __syncthreads();
        const int nmoves = C.nres;
        long long npairs = 0;
        uint4* Fc = F + C.atom0;
        ulonglong4_32a* Mc = M + C.atom0;
        int mv = 0, buf = 0;
        unsigned prev_acc = 0;                 // accepted moves of the previous iteration (records P[buf ^ 1])
        // moves left before the next dmax adjustment of each type (0: the type is never adjusted)
        const bool adjust = C.each[0] > 0 || C.each[1] > 0;
        int to_adj[2];
#pragma unroll
        for (int t = 0; t < 2; t++) to_adj[t] = C.each[t] > 0 ? C.each[t] - (int)(S.moves % (unsigned long long)C.each[t]) : 0;
        float eh = 0.0f, el = 0.0f;            // accepted dE of this sweep (float-float, warp 0 lane 0)
        while (mv < nmoves) {
            int kk = min(K, nmoves - mv);
            if (adjust) {   // an iteration ends at the move after which dmax is adjusted
#pragma unroll
                for (int t = 0; t < 2; t++) if (to_adj[t] > 0) kk = min(kk, to_adj[t]);
            }
            const bool gact = grp < kk;
            MoveRec<A>* R = P[buf ^ 1];
            if (tid < KM) { s_cm[buf][tid] = 0u; s_sr[buf][tid] = 0u; }
            float acc = 0.0f;
            int np = 0;
            if (gact) {
                // ---- the move of my group (every warp of the group, lanes = atoms)
                const unsigned long long cg = S.moves + (unsigned long long)(mv + grp);
                const U4 q0 = philox4x32_10(U4{(uint32_t)cg, (uint32_t)(cg >> 32), (uint32_t)c, 0u}, C.key0, C.key1);
                const U4 q1 = philox4x32_10(U4{(uint32_t)cg, (uint32_t)(cg >> 32), (uint32_t)c, 1u}, C.key0, C.key1);
                const int res = (int)(((uint64_t)q0.y * (uint64_t)C.nres) >> 32);
                const bool rot = C.ntypes_move == 2 && (q0.x & 1u);
                const int piv = (int)(((uint64_t)q0.z * (uint64_t)apr) >> 32);
                const int k = lane < apr ? lane : 0;
                const int a = res * apr + k;
                // lanes take list entries (neighbour residues), CH per lane in flight, each with all
                // of its atoms.  The neighbour indices of each chunk are loaded one chunk ahead (the
                // first ones before the move is formed, so their latency overlaps the moved
                // residue's loads and the move arithmetic): a chunk waits for its position loads
                // only, not for an index load and then the positions.
                constexpr int CH = A >= 3 ? 1 : (A == 2 ? 2 : 4);
                const uint16_t* row = LST + (size_t)(C.res0 + res) * G.cap;
                const int nent = NL[C.res0 + res];
                int qn[CH];
#pragma unroll
                for (int u = 0; u < CH; u++) {
                    const int e = gw * 32 + u * GS + lane;
                    qn[u] = e < G.cap ? row[e] : 0;
                }
                uint4 fo = Fc[a];
                ulonglong4_32a mo = Mc[a];
                const uint4 fb = FB[C.atom0 + a];
                // records of the previous iteration: accepted moves whose commits may not have landed
                unsigned sub = 0;
                for (unsigned pm = prev_acc; pm; pm &= pm - 1) {
                    const int h = __ffs(pm) - 1;
                    if (R[h].res == res) {
                        fo = R[h].fn[k];
                        mo = make_ulonglong4_32a(R[h].mn[k][0], R[h].mn[k][1], R[h].mn[k][2], 0ull);
                    }
                }
                const uint4 fo0 = make_uint4(__shfl_sync(0xffffffffu, fo.x, 0), __shfl_sync(0xffffffffu, fo.y, 0),
                                             __shfl_sync(0xffffffffu, fo.z, 0), 0u);
                for (unsigned pm = prev_acc; pm; pm &= pm - 1) {
                    const int h = __ffs(pm) - 1;
                    const float dx = fdelta(fo0.x, R[h].fo0.x, Ls0, Ll0), dy = fdelta(fo0.y, R[h].fo0.y, Ls1, Ll1),
                                dz = fdelta(fo0.z, R[h].fo0.z, Ls2, Ll2);
                    if (dx * dx + dy * dy + dz * dz <= G.subst2) sub |= 1u << h;
                }
                const float ct = 2.0f * u01f(q0.w) - 1.0f;   // uniform direction: cos(theta), phi
                const float st = sqrtf(fmaxf(0.0f, 1.0f - ct * ct));
                float sphi, cphi;
                sincospif(2.0f * u01f(q1.x), &sphi, &cphi);
                const float ux = st * cphi, uy = st * sphi, uz = ct;
                float dx, dy, dz;
                if (!rot) {
                    const float rad = (float)S.dmax[0] * cbrtf(u01f(q1.y));
                    dx = rad * ux; dy = rad * uy; dz = rad * uz;
                } else {
                    // unit quaternion for an angle uniform in [-dmax, dmax] degrees about u;
                    // rotated offset minus offset = 2 q_w (q_v x o) + 2 q_v x (q_v x o)
                    const uint32_t px = __shfl_sync(0xffffffffu, fo.x, piv), py = __shfl_sync(0xffffffffu, fo.y, piv),
                                   pz = __shfl_sync(0xffffffffu, fo.z, piv);
                    float sh, ch;
                    sincospif((float)S.dmax[1] * (2.0f * u01f(q1.y) - 1.0f) * (1.0f / 360.0f), &sh, &ch);
                    const float qw = ch, qx = sh * ux, qy = sh * uy, qz = sh * uz;
                    const float ox = fdelta(px, fo.x, Ls0, Ll0), oy = fdelta(py, fo.y, Ls1, Ll1),
                                oz = fdelta(pz, fo.z, Ls2, Ll2);
                    const float tx = 2.0f * (qy * oz - qz * oy), ty = 2.0f * (qz * ox - qx * oz), tz = 2.0f * (qx * oy - qy * ox);
                    dx = qw * tx + (qy * tz - qz * ty);
                    dy = qw * ty + (qz * tx - qx * tz);
                    dz = qw * tz + (qx * ty - qy * tx);
                }
                const unsigned long long nx = mo.x + master_step(dx, C.tofix32[0]);
                const unsigned long long ny = mo.y + master_step(dy, C.tofix32[1]);
                const unsigned long long nz = mo.z + master_step(dz, C.tofix32[2]);
                const uint4 fn = make_uint4((uint32_t)(nx >> 32), (uint32_t)(ny >> 32), (uint32_t)(nz >> 32), fo.w);
                const float mx = fdelta(fo.x, fn.x, Ls0, Ll0), my = fdelta(fo.y, fn.y, Ls1, Ll1),
                            mz = fdelta(fo.z, fn.z, Ls2, Ll2);
                const float ofx = fdelta(fo0.x, fo.x, Ls0, Ll0), ofy = fdelta(fo0.y, fo.y, Ls1, Ll1),
                            ofz = fdelta(fo0.z, fo.z, Ls2, Ll2);
                if (gw == 0) {
                    // alpha >= ahi / 2^32 and below it by < 2^-32: for ahi >= 2^16 the FP32
                    // -ln(alpha) is within 2e-5 of the exact one, inside the decision margin
                    const float lna = q1.z >= 65536u ? -__logf(__uint2float_rn(q1.z) * 2.3283064365386963e-10f)
                                                     : __int_as_float(0x7fc00000);
                    for (int cp = 0; cp < CL; cp++) {
                        MoveRec<A>& Q = cp ? *peer(&P[buf][grp]) : P[buf][grp];
                        if (lane < apr) {
                            Q.fn[lane] = fn;
                            Q.fo[lane] = fo;
                            Q.mn[lane][0] = nx; Q.mn[lane][1] = ny; Q.mn[lane][2] = nz;
                            Q.fb[lane] = fb;
                        }
                        if (lane == 0) {
                            Q.fo0 = fo0;
                            Q.res = res;
                            Q.rot = rot ? 1 : 0;
                            Q.ahi = q1.z;
                            Q.alo = q1.w;
                            Q.lna = lna;
                        }
                    }
                }
                float m[A][3], off[A][3];
#pragma unroll
                for (int j = 0; j < A; j++) {
                    m[j][0] = __shfl_sync(0xffffffffu, mx, j); m[j][1] = __shfl_sync(0xffffffffu, my, j);
                    m[j][2] = __shfl_sync(0xffffffffu, mz, j);
                    off[j][0] = __shfl_sync(0xffffffffu, ofx, j); off[j][1] = __shfl_sync(0xffffffffu, ofy, j);
                    off[j][2] = __shfl_sync(0xffffffffu, ofz, j);
                }
                const bool wrap = C.wrap_offsets != 0;
                // prefilter radius of this move: a neighbour atom b has a pair within rc of atom j,
                // before or after the move, only if |b - c| <= rc + max_j |a_j - c| + max_j |m_j|
                // (c: the residue's centroid before the move; its first atom in small boxes, where
                // only displacements from the first atom are minimum images)
                float cx = 0.0f, cy = 0.0f, cz = 0.0f, skip2;
                {
                    if (!wrap) {
#pragma unroll
                        for (int j = 1; j < A; j++)
                            if (j < apr) { cx += off[j][0]; cy += off[j][1]; cz += off[j][2]; }
                        const float ia = 1.0f / (float)apr;
                        cx *= ia; cy *= ia; cz *= ia;
                    }
                    float ext2 = 0.0f, mv2 = 0.0f;
#pragma unroll
                    for (int j = 0; j < A; j++)
                        if (j < apr) {
                            const float dx = off[j][0] - cx, dy = off[j][1] - cy, dz = off[j][2] - cz;
                            ext2 = fmaxf(ext2, dx * dx + dy * dy + dz * dz);
                            mv2 = fmaxf(mv2, m[j][0] * m[j][0] + m[j][1] * m[j][1] + m[j][2] * m[j][2]);
                        }
                    const float rs = rcf + sqrtf(ext2) + sqrtf(mv2) + 1e-3f;
                    skip2 = rs * rs;
                }
                // ---- neighbour atoms: compaction into the ring, evaluation 32 at a time
                auto eval = [&](const float4 v) {
                    const uint32_t w = __float_as_uint(v.w);
#pragma unroll
                    for (int j = 0; j < A; j++) {
                        if (j >= apr) break;
                        const float4 tb = s_tab[j][w];
                        // b - a_j = (b - a_0) - (a_j - a_0), back to the minimum image in small boxes
                        float ex = j ? v.x - off[j][0] : v.x;
                        float ey = j ? v.y - off[j][1] : v.y;
                        float ez = j ? v.z - off[j][2] : v.z;
                        if (wrap) {
                            ex -= (ex > C.Lhalf[0]) ? C.Lf[0] : ((ex < -C.Lhalf[0]) ? -C.Lf[0] : 0.0f);
                            ey -= (ey > C.Lhalf[1]) ? C.Lf[1] : ((ey < -C.Lhalf[1]) ? -C.Lf[1] : 0.0f);
                            ez -= (ez > C.Lhalf[2]) ? C.Lf[2] : ((ez < -C.Lhalf[2]) ? -C.Lf[2] : 0.0f);
                        }
                        // d_old = b - a_old, d_new = b - a_new = d_old - m
                        acc += pair_delta<PK>(ex, ey, ez, m[j][0], m[j][1], m[j][2], tb.x, tb.y, tb.z, c2f, n2f,
                                                        k3f, np);
                    }
                };
                int head = 0, tail = 0;
                for (int base = gw * 32; base < nent; base += CH * GS) {
                    int q[CH];
                    uint4 pb[CH][A];
#pragma unroll
                    for (int u = 0; u < CH; u++) q[u] = base + u * GS + lane < nent ? qn[u] : -1;
#pragma unroll
                    for (int u = 0; u < CH; u++)
#pragma unroll
                        for (int b = 0; b < A; b++)
                            pb[u][b] = (q[u] >= 0 && b < apr) ? Fc[q[u] * apr + b] : make_uint4(0, 0, 0, 0);
#pragma unroll
                    for (int u = 0; u < CH; u++) {   // the next chunk's indices
                        const int e = base + CH * GS + u * GS + lane;
                        qn[u] = e < nent ? (int)row[e] : 0;
                    }
#pragma unroll
                    for (int u = 0; u < CH; u++) {
                        if (base + u * GS >= nent) break;
                        if (sub) {
                            for (unsigned pm = sub; pm; pm &= pm - 1) {
                                const int h = __ffs(pm) - 1;
                                if (q[u] == R[h].res) {
#pragma unroll
                                    for (int b = 0; b < A; b++)
                                        if (b < apr) pb[u][b] = R[h].fn[b];
                                }
                            }
                        }
                        // each atom of the entry is kept on its own distance from the moved
                        // residue's first atom
#pragma unroll
                        for (int b = 0; b < A; b++) {
                            if (b >= apr) break;
                            const float ex = fdelta(fo0.x, pb[u][b].x, Ls0, Ll0), ey = fdelta(fo0.y, pb[u][b].y, Ls1, Ll1),
                                        ez = fdelta(fo0.z, pb[u][b].z, Ls2, Ll2);
                            const float ux = ex - cx, uy = ey - cy, uz = ez - cz;
                            const bool keep = q[u] >= 0 && ux * ux + uy * uy + uz * uz <= skip2;
                            const unsigned bal = __ballot_sync(0xffffffffu, keep);
                            if (keep)
                                ring[(head + __popc(bal & lt_mask)) & (RING - 1)] = make_float4(ex, ey, ez, __uint_as_float(pb[u][b].w));
                            head += __popc(bal);
                            if (head - tail >= 32) {
                                __syncwarp();
                                eval(ring[(tail + lane) & (RING - 1)]);
                                tail += 32;
                                __syncwarp();
                            }
                        }
                    }
                }
                __syncwarp();
                if (lane < head - tail) eval(ring[(tail + lane) & (RING - 1)]);
                __syncwarp();
            }
            // float-float warp reduction (TwoSum) of the warp's share of its move's dE
            float hi = acc, lo = 0.0f;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                const float oh = __shfl_xor_sync(0xffffffffu, hi, o), ol = __shfl_xor_sync(0xffffffffu, lo, o);
                float sm, e;
                two_sum(hi, oh, sm, e);
                hi = sm;
                lo = lo + ol + e;
            }
            if (lane == 0) {
                s_red[buf][rank * NW + warp] = make_float2(hi, lo);
                if (CL > 1) *peer(&s_red[buf][rank * NW + warp]) = make_float2(hi, lo);
            }
            unit_sync();
            // ---- decisions, identical in every warp: lane g < kk holds move g
            const MoveRec<A>* Q = P[buf];
            float deh = 0.0f, del = 0.0f;           // dE of move `lane` as a float-float pair
            bool acc_raw = false;
            {
                // lane = g * WPG + w holds warp w's partial of move g; segmented butterfly over w
                float2 v = lane < CL * NW ? s_red[buf][lane] : make_float2(0.0f, 0.0f);
                for (int o = 1; o < WPG; o <<= 1) {
                    const float oh = __shfl_xor_sync(0xffffffffu, v.x, o), ol = __shfl_xor_sync(0xffffffffu, v.y, o);
                    float sm, e;
                    two_sum(v.x, oh, sm, e);
                    v.x = sm;
                    v.y = v.y + ol + e;
                }
                const int src = (lane < kk ? lane : 0) * WPG;
                deh = __shfl_sync(0xffffffffu, v.x, src);
                del = __shfl_sync(0xffffffffu, v.y, src);
            }
            // Interaction masks and dE corrections of the iteration's moves (the records are in this
            // CTA's shared memory): for move g, the earlier moves h that moved its residue (s_sr) or
            // may interact with it (first atoms within rc + 2 extents + 2 largest moves, s_cm), and
            // for each of the latter the change of the pair terms between the two residues
            // (pair_correction), needed if h is accepted.  Pair (g, h < g), p = g (g - 1) / 2 + h, is
            // tested by lane p / NW of warp p % NW, so the tests and the corrections of the near
            // pairs (computed by the whole warp, one at a time) spread evenly over the warps.
            {
                const int npr = kk * (kk - 1) / 2;
                for (int p0 = 0; p0 < npr; p0 += 32 * NW) {
                    const int p = p0 + lane * NW + warp;
                    int g = 0, h = 0;
                    bool same = false, near = false;
                    if (p < npr) {
                        g = (int)(0.5f * (1.0f + sqrtf(1.0f + 8.0f * (float)p)));
                        if (g * (g - 1) / 2 > p) g--;
                        else if ((g + 1) * g / 2 <= p) g++;
                        h = p - g * (g - 1) / 2;
                        same = Q[h].res == Q[g].res;
                        if (!same) {
                            const float dx = fdelta(Q[h].fo0.x, Q[g].fo0.x, Ls0, Ll0);
                            const float dy = fdelta(Q[h].fo0.y, Q[g].fo0.y, Ls1, Ll1);
                            const float dz = fdelta(Q[h].fo0.z, Q[g].fo0.z, Ls2, Ll2);
                            near = dx * dx + dy * dy + dz * dz <= G.indep2;
                        }
                    }
                    if (same) atomicOr(&s_sr[buf][g], 1u << h);
                    if (near) atomicOr(&s_cm[buf][g], 1u << h);
                    for (unsigned nb = __ballot_sync(0xffffffffu, near); nb; nb &= nb - 1) {
                        const int l = __ffs(nb) - 1;
                        const int gg = __shfl_sync(0xffffffffu, g, l), hh = __shfl_sync(0xffffffffu, h, l);
                        float ch = pair_correction<A, PK>(Q[gg], Q[hh], apr, lane, s_tab, Ls0, Ls1, Ls2, Ll0, Ll1, Ll2, c2f, n2f, k3f);
                        float cl = 0.0f;
#pragma unroll
                        for (int o = 16; o > 0; o >>= 1) {
                            const float oh = __shfl_xor_sync(0xffffffffu, ch, o), ol = __shfl_xor_sync(0xffffffffu, cl, o);
                            float sm, e;
                            two_sum(ch, oh, sm, e);
                            ch = sm;
                            cl = cl + ol + e;
                        }
                        if (lane == 0) s_corr[gg][hh] = make_float2(ch, cl);
                    }
                }
            }
            __syncthreads();
            if (lane < kk) acc_raw = metropolis_accept(deh, del, Q[lane], C.beta_f, C.beta);
            // In move order: move g stands unless an earlier accepted move of the iteration moved
            // its residue.  Its dE was evaluated against the chain before the iteration; each
            // earlier accepted move h that may interact with it changes only the pair terms
            // between the two residues, so dE is corrected by those terms and the test is taken
            // again on the corrected value: the dE and decision of the sequential chain, up to FP32
            // summation order.
            unsigned araw = __ballot_sync(0xffffffffu, acc_raw);
            unsigned accmask = 0;
            int ng = kk;
            for (int g = 0; g < kk; g++) {
                if (s_sr[buf][g] & accmask) { ng = g; break; }
                const unsigned cset = s_cm[buf][g] & accmask;
                if (cset) {                          // warp-uniform
                    if (lane == g) {
                        for (unsigned hm = cset; hm; hm &= hm - 1) {
                            const float2 c = s_corr[g][__ffs(hm) - 1];
                            float sm, e;
                            two_sum(deh, c.x, sm, e);
                            deh = sm;
                            del = del + c.y + e;
                        }
                        acc_raw = metropolis_accept(deh, del, Q[g], C.beta_f, C.beta);
                    }
                    araw = __ballot_sync(0xffffffffu, acc_raw);
                }
                accmask |= araw & (1u << g);
            }
            // far check of the accepted moves (t = g * apr + j over the lanes) and the commits
            bool far = false;
            {
                float e2 = 0.0f;
                for (int t = lane; t < ng * apr; t += 32) {
                    const int g = t / apr, j = t - g * apr;
                    if ((accmask >> g) & 1u) {
                        const float ex = fdelta(Q[g].fb[j].x, Q[g].fn[j].x, Ls0, Ll0);
                        const float ey = fdelta(Q[g].fb[j].y, Q[g].fn[j].y, Ls1, Ll1);
                        const float ez = fdelta(Q[g].fb[j].z, Q[g].fn[j].z, Ls2, Ll2);
                        const float d2 = ex * ex + ey * ey + ez * ez;
                        e2 = fmaxf(e2, d2);
                        far = far || d2 > G.half_skin2;
                    }
                }
                if (warp == 0) {
                    for (int o = 16; o > 0; o >>= 1) e2 = fmaxf(e2, __shfl_xor_sync(0xffffffffu, e2, o));
                    S.maxd2 = fmaxf(S.maxd2, e2);
                }
            }
            if (gw == 0 && grp < ng && ((accmask >> grp) & 1u) && lane < apr) {   // commit: atom = lane
                const int a = Q[grp].res * apr + lane;
                Mc[a] = make_ulonglong4_32a(Q[grp].mn[lane][0], Q[grp].mn[lane][1], Q[grp].mn[lane][2], 0ull);
                Fc[a] = Q[grp].fn[lane];
            }
            if (mlog && rank == 0 && warp == 0) {   // logged sweep: the standing moves in chain order
                MoveLogDev* lg = mlog + C.res0 + mv;
                for (int t = lane; t < ng * apr; t += 32) {
                    const int g = t / apr, j = t - g * apr;
                    lg[g].pos[j][0] = Q[g].mn[j][0];
                    lg[g].pos[j][1] = Q[g].mn[j][1];
                    lg[g].pos[j][2] = Q[g].mn[j][2];
                }
                if (lane < ng) {
                    lg[lane].de = (double)deh + (double)del;
                    lg[lane].res = Q[lane].res;
                    lg[lane].flags = Q[lane].rot | (int)(((accmask >> lane) & 1u) << 1);
                    lg[lane].ahi = Q[lane].ahi;
                    lg[lane].alo = Q[lane].alo;
                }
            }
            if (grp < ng) npairs += np;
            if (adjust) {   // dmax adjustment after the standing moves, in move order (every thread alike)
                for (int g = 0; g < ng; g++) {
                    if ((accmask >> g) & 1u) S.acc_tmp[Q[g].rot]++;
#pragma unroll
                    for (int t = 0; t < 2; t++) {
                        if (to_adj[t] > 0 && --to_adj[t] == 0) {
                            const double ratio = (double)S.acc_tmp[t] / (double)C.each[t];
                            S.dmax[t] = fmin(C.dmax_cap[t], S.dmax[t] * (ratio > C.target[t] ? 1.10 : 0.9));
                            S.acc_tmp[t] = 0;
                            to_adj[t] = C.each[t];
                        }
                    }
                }
            }
            if (warp == 0) {   // statistics and the sweep's energy change, in move order
                for (int g = 0; g < ng; g++) {
                    const float dh = __shfl_sync(0xffffffffu, deh, g), dl = __shfl_sync(0xffffffffu, del, g);
                    if (lane == 0) {
                        S.trials++;
                        if ((accmask >> g) & 1u) {
                            S.accepted++;
                            float sm, e;
                            two_sum(eh, dh, sm, e);
                            eh = sm;
                            el = el + dl + e;
                        }
                    }
                }
            }
            mv += ng;
            prev_acc = accmask;
            buf ^= 1;
            if (__any_sync(0xffffffffu, far)) {   // identical in every warp
                unit_sync();                      // the commits have landed
                if (rank == 0)
                    chain_rebuild<APR>(C, G, F, FB, LST, NL, s_cell, g_order + C.res0, g_cell + C.res0, g_pos + C.res0,
                                       &s_err, reinterpret_cast<uint4*>(ring));
                if (CL > 1) unit_sync();          // CTA 1 waits for CTA 0's lists
                if (tid == 0) { S.rebuilds++; S.maxd2 = 0.0f; }
                prev_acc = 0;
            }
        }
        __syncthreads();
        for (int o = 16; o > 0; o >>= 1) npairs += __shfl_xor_sync(0xffffffffu, npairs, o);
        if (lane == 0) atomicAdd(rank == 0 ? &s_pairs : peer(&s_pairs), (unsigned long long)npairs);
        unit_sync();
        if (rank == 0 && tid == 0) {
            S.etot += (double)eh + (double)el;
            S.pairs += (long long)s_pairs;
            S.moves += (unsigned long long)nmoves;
            if (s_err) S.err = s_err;
            state[c] = S;
        }
    }  // chains of this CTA
}

// FP64 view of a master coordinate
__device__ __forceinline__ double master_to_f64(unsigned long long v, double L) {
    return (double)(long long)v * (L * (1.0 / TWO64));
}

// ---- fresh FP64 energy of every chain (reference arithmetic, all pairs, cutoff + switch)
constexpr int ETILE = 128;
__global__ void k_batch_energy64(const ChainDev* __restrict__ chains, const int* __restrict__ tile_chain,
                                 const int* __restrict__ tile_first, const ulonglong4_32a* __restrict__ M,
                                 const double* __restrict__ prm, CutDev cut, double* part) {
    const int t = blockIdx.x;
    const int c = tile_chain[t];
    const ChainDev& C = chains[c];
    const int n = C.nres * C.apr;
    const int i = tile_first[t] + threadIdx.x;
    double s = 0.0;
    if (i < n) {
        PbcDev pbc;
        pbc.type = 2;
        for (int k = 0; k < 3; k++) { pbc.L[k] = C.L[k]; pbc.rL[k] = C.rL[k]; }
        const ulonglong4_32a ma = M[C.atom0 + i];
        const double ax = master_to_f64(ma.x, C.L[0]), ay = master_to_f64(ma.y, C.L[1]), az = master_to_f64(ma.z, C.L[2]);
        const int ri = i / C.apr;
        const double* pa = prm + 3 * (size_t)(C.atom0 + i);
        for (int j = i + 1; j < n; j++) {
            if (j / C.apr == ri) continue;  // intra-residue pairs are excluded
            const ulonglong4_32a mb = M[C.atom0 + j];
            const double r2 = ref64_dist2(ax, ay, az, master_to_f64(mb.x, C.L[0]), master_to_f64(mb.y, C.L[1]),
                                          master_to_f64(mb.z, C.L[2]), pbc);
            if (r2 > cut.c2) continue;
            const double* pb = prm + 3 * (size_t)(C.atom0 + j);
            double el, vd;
            ref64_pair(r2, pa[0], pb[0], pa[1], pb[1], pa[2], pb[2], true, cut, el, vd);
            s += CHGCHARMM * KCALTOIU * el + 4.0 * vd;
        }
    }
    s = warp_sum(s);
    __shared__ double sh[ETILE / 32];
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double v = 0.0;
        for (int w = 0; w < ETILE / 32; w++) v += sh[w];
        part[t] = v;
    }
}

// ---- mixed-precision energy of every chain over its neighbour lists (each pair once: q > r)
// One warp per residue over the GPU writes the residue's share; one block per chain then sums the
// shares in residue order, so the result does not depend on scheduling.
template <int APR>
__global__ void __launch_bounds__(256) k_batch_energy_res(const ChainDev* __restrict__ chains, BatchGeom G,
                                                          const uint4* __restrict__ F, const int* __restrict__ res_chain,
                                                          const uint16_t* __restrict__ LST, const int* __restrict__ NL,
                                                          double* e_res, int64_t nres_total, const int* __restrict__ only,
                                                          const int* __restrict__ any) {
    if (any && !*any) return;   // a masked recompute with no chain to recompute
    // A warp per residue r.  Lanes scan r's list 32 entries at a time; the entries q > r whose
    // first atom lies within rc + 2 extents of r's are compacted into the warp's ring in shared
    // memory, and each time 32 are pending every lane evaluates one residue pair: all atom pairs
    // of (r, q), with r's atoms in registers.  Atom pairs beyond rc take r^2 = rc^2, where the
    // switch is exactly 0 (no divergent skip).  Coulomb and LJ are summed per lane as float-float
    // pairs (TwoSum), so the result does not depend on the list order beyond ~1e-14; the warp
    // sums in FP64.
    constexpr int A = APR ? APR : MAX_APR;
    constexpr int ERING = 64;
    __shared__ int s_q[8][ERING];
    CutDev cut;
    cut.mode = 1; cut.c2 = 0; cut.n2 = 0; cut.sw2 = 0;
    cut.c2f = G.c2f; cut.n2f = G.n2f; cut.sw2f = G.sw2f;
    const float c2 = G.c2f;
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const unsigned lt_mask = (1u << lane) - 1u;
    int* ring = s_q[wib];
    const int64_t warps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t gr = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; gr < nres_total; gr += warps) {
        const int c = res_chain[gr];
        if (only && !only[c]) continue;    // a chain whose energy is not asked for
        const ChainDev& C = chains[c];
        if (APR && C.apr != APR) continue;
        const int apr = APR ? APR : C.apr;
        const int r = (int)(gr - C.res0);
        const uint4* Fc = F + C.atom0;
        const uint16_t* row = LST + (size_t)gr * G.cap;
        const int nl = NL[gr];
        const float Ls0 = C.Ls[0], Ls1 = C.Ls[1], Ls2 = C.Ls[2], Ll0 = C.Lsl[0], Ll1 = C.Lsl[1], Ll2 = C.Lsl[2];
        uint4 pa[A];
#pragma unroll
        for (int k = 0; k < A; k++) pa[k] = k < apr ? Fc[r * apr + k] : make_uint4(0, 0, 0, 0);
        // r's atoms as offsets from its first atom: an atom pair's displacement is then the exact
        // fixed-point displacement of q's atom from r's first atom minus r's offset, brought back
        // to the minimum image in boxes small enough to need it
        float ro[A][3];
#pragma unroll
        for (int k = 0; k < A; k++) {
            ro[k][0] = fdelta(pa[0].x, pa[k].x, Ls0, Ll0);
            ro[k][1] = fdelta(pa[0].y, pa[k].y, Ls1, Ll1);
            ro[k][2] = fdelta(pa[0].z, pa[k].z, Ls2, Ll2);
        }
        const bool wrap = C.wrap_offsets != 0;
        float eh = 0.0f, elo = 0.0f, vh = 0.0f, vlo = 0.0f;
        // residue q (>= 0) against r, by this lane
        auto eval = [&](int q) {
            uint4 pb[A];
#pragma unroll
            for (int b = 0; b < A; b++) pb[b] = b < apr ? Fc[q * apr + b] : make_uint4(0, 0, 0, 0);
            float d0[A][3];
#pragma unroll
            for (int b = 0; b < A; b++) {
                d0[b][0] = fdelta(pa[0].x, pb[b].x, Ls0, Ll0);
                d0[b][1] = fdelta(pa[0].y, pb[b].y, Ls1, Ll1);
                d0[b][2] = fdelta(pa[0].z, pb[b].z, Ls2, Ll2);
            }
#pragma unroll
            for (int k = 0; k < A; k++) {
                if (k >= apr) break;
#pragma unroll
                for (int b = 0; b < A; b++) {
                    if (b >= apr) break;
                    float dx = d0[b][0] - ro[k][0], dy = d0[b][1] - ro[k][1], dz = d0[b][2] - ro[k][2];
                    if (wrap) {
                        dx -= (dx > C.Lhalf[0]) ? C.Lf[0] : ((dx < -C.Lhalf[0]) ? -C.Lf[0] : 0.0f);
                        dy -= (dy > C.Lhalf[1]) ? C.Lf[1] : ((dy < -C.Lhalf[1]) ? -C.Lf[1] : 0.0f);
                        dz -= (dz > C.Lhalf[2]) ? C.Lf[2] : ((dz < -C.Lhalf[2]) ? -C.Lf[2] : 0.0f);
                    }
                    const float u = fminf(fmaf(dx, dx, fmaf(dy, dy, dz * dz)), c2);
                    // slot k of r against slot b of q (F.w holds the slot); float-float charge and
                    // LJ constants: per-type roundings of the products are systematic biases that
                    // the cancellation in the total would amplify
                    float el, vd;
                    mixed_pair(u, C.tab[k][b][0], C.tab[k][b][3], C.tab[k][b][1], C.tab[k][b][2], true, cut, el, vd,
                               C.tablo[k][b][0], C.tablo[k][b][1]);
                    float sm, er;
                    two_sum(eh, el, sm, er);
                    eh = sm;
                    elo += er;
                    two_sum(vh, vd, sm, er);
                    vh = sm;
                    vlo += er;
                }
            }
        };
        int head = 0, tail = 0;
        for (int e0 = 0; e0 < nl; e0 += 32) {
            const int e = e0 + lane;
            const int q = e < nl ? (int)row[e] : -1;
            bool keep = false;
            if (q > r) {
                // first atoms farther than rc + 2 extents: no atom pair of the two residues is within rc
                const uint4 q0 = Fc[q * apr];
                const float dx = fdelta(pa[0].x, q0.x, Ls0, Ll0), dy = fdelta(pa[0].y, q0.y, Ls1, Ll1),
                            dz = fdelta(pa[0].z, q0.z, Ls2, Ll2);
                keep = fmaf(dx, dx, fmaf(dy, dy, dz * dz)) <= G.pair2;
            }
            const unsigned bal = __ballot_sync(0xffffffffu, keep);
            if (keep) ring[(head + __popc(bal & lt_mask)) & (ERING - 1)] = q;
            head += __popc(bal);
            if (head - tail >= 32) {
                __syncwarp();
                eval(ring[(tail + lane) & (ERING - 1)]);
                tail += 32;
            }
            __syncwarp();
        }
        if (lane < head - tail) eval(ring[(tail + lane) & (ERING - 1)]);
        __syncwarp();
        // float-float butterfly over the lanes (GB300's FP64 rate is 1/64 of FP32); lane 0 adds the
        // two parts in FP64
        float th, tl;
        two_sum(eh, vh, th, tl);
        tl += elo + vlo;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const float oh = __shfl_xor_sync(0xffffffffu, th, o), ol = __shfl_xor_sync(0xffffffffu, tl, o);
            float sm, er;
            two_sum(th, oh, sm, er);
            th = sm;
            tl = tl + ol + er;
        }
        if (lane == 0) e_res[gr] = (double)th + (double)tl;
    }
}

__global__ void k_batch_energy_sum(const ChainDev* __restrict__ chains, const double* __restrict__ e_res,
                                   ChainState* state, int nchains, const int* __restrict__ only,
                                   const int* __restrict__ any) {
    __shared__ double sh[256];
    if (any && !*any) return;
    const int c = blockIdx.x;
    if (c >= nchains || (only && !only[c])) return;
    const ChainDev& C = chains[c];
    double s = 0.0;
    for (int r = threadIdx.x; r < C.nres; r += blockDim.x) s += e_res[C.res0 + r];
    sh[threadIdx.x] = s;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) state[c].etot = sh[0];
}

// FP64 coordinates (all chains concatenated) -> 64-bit masters and 32-bit mirrors
// The chain's largest squared displacement from its list-build positions FB enters state.maxd2, so
// the next list build (k_batch_bin) rebuilds exactly the chains whose imported atoms moved beyond
// the rebuild threshold.  Launched with 256 threads per chain.
// An atom whose three input coordinates equal the FP64 view of its current master (what
// k_batch_export gave out) keeps its master: a chain whose atoms all come back unchanged is left
// exactly as it was (changed[c] = 0), and its running energy stands.  changed[nchains] becomes 1
// when any chain changed; changed[] is zeroed before the launch.  Grid: chains x slices of 256
// atoms (a chain's slices stride over its atoms).
__global__ void __launch_bounds__(256) k_batch_import(const ChainDev* __restrict__ chains, const double* __restrict__ xyz,
                                                      int64_t natoms, ulonglong4_32a* M, uint4* F,
                                                      const uint4* __restrict__ FB, ChainState* state, int* changed,
                                                      int nchains) {
    __shared__ float s_max[8];
    __shared__ int s_changed;
    const int c = blockIdx.x;
    if (c >= nchains) return;
    const ChainDev& C = chains[c];
    const int n = C.nres * C.apr;
    if ((int)(blockIdx.y * blockDim.x) >= n) return;   // a slice past the chain's atoms (block-uniform)
    if (threadIdx.x == 0) s_changed = 0;
    __syncthreads();
    float dmax = 0.0f;
    for (int i = blockIdx.y * blockDim.x + threadIdx.x; i < n; i += gridDim.y * blockDim.x) {
        const int64_t a = C.atom0 + i;
        const ulonglong4_32a mo = M[a];
        const double v[3] = {xyz[a], xyz[natoms + a], xyz[2 * natoms + a]};
        if (v[0] == master_to_f64(mo.x, C.L[0]) && v[1] == master_to_f64(mo.y, C.L[1]) && v[2] == master_to_f64(mo.z, C.L[2]))
            continue;
        s_changed = 1;
        unsigned long long m[3];
        for (int k = 0; k < 3; k++) {
            double u = v[k] * C.rL[k];
            u -= rint(u);
            if (u >= 0.5) u -= 1.0;
            m[k] = (unsigned long long)__double2ll_rn(u * TWO64);
        }
        M[a] = make_ulonglong4_32a(m[0], m[1], m[2], 0ull);
        const uint4 f = make_uint4((uint32_t)(m[0] >> 32), (uint32_t)(m[1] >> 32), (uint32_t)(m[2] >> 32), (uint32_t)(i % C.apr));
        F[a] = f;
        const uint4 fb = FB[a];
        const float ex = fdelta(fb.x, f.x, C.Ls[0], C.Lsl[0]), ey = fdelta(fb.y, f.y, C.Ls[1], C.Lsl[1]),
                    ez = fdelta(fb.z, f.z, C.Ls[2], C.Lsl[2]);
        dmax = fmaxf(dmax, fmaf(ex, ex, fmaf(ey, ey, ez * ez)));
    }
    for (int o = 16; o > 0; o >>= 1) dmax = fmaxf(dmax, __shfl_xor_sync(0xffffffffu, dmax, o));
    if ((threadIdx.x & 31) == 0) s_max[threadIdx.x >> 5] = dmax;
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < (int)(blockDim.x >> 5); w++) dmax = fmaxf(dmax, s_max[w]);
        // non-negative floats order as their bit patterns
        atomicMax(reinterpret_cast<int*>(&state[c].maxd2), __float_as_int(dmax));
        if (s_changed) {
            atomicOr(&changed[c], 1);
            atomicOr(&changed[nchains], 1);
        }
    }
}

__global__ void k_batch_export(const ChainDev* __restrict__ chains, const ulonglong4_32a* __restrict__ M, int64_t natoms,
                               double* xyz, int nchains) {
    const int c = blockIdx.x;
    if (c >= nchains) return;
    const ChainDev& C = chains[c];
    const int n = C.nres * C.apr;
    for (int i = blockIdx.y * blockDim.x + threadIdx.x; i < n; i += gridDim.y * blockDim.x) {
        const int64_t a = C.atom0 + i;
        const ulonglong4_32a m = M[a];
        xyz[a] = master_to_f64(m.x, C.L[0]);
        xyz[natoms + a] = master_to_f64(m.y, C.L[1]);
        xyz[2 * natoms + a] = master_to_f64(m.z, C.L[2]);
    }
}

}  // namespace mcg

// ==============================================================================================
using namespace mcg;

static uint64_t host_master(double v, double rL) {
    double u = v * rL;
    u -= std::nearbyint(u);          // [-0.5, 0.5]
    if (u >= 0.5) u -= 1.0;
    return (uint64_t)(int64_t)std::llrint(u * TWO64);
}

static double host_view(uint64_t v, double L) { return (double)(int64_t)v * (L / TWO64); }

static int balloc_d(double** p, size_t n) {
    cudaError_t e = cudaMalloc((void**)p, std::max<size_t>(1, n) * sizeof(double));
    if (e != cudaSuccess) return fail(MCG_ECUDA, std::string("cudaMalloc: ") + cudaGetErrorString(e));
    return MCG_OK;
}

struct mcg_batch {
    int nchains = 0;
    int64_t natoms = 0, nres = 0;
    int apr_all = 0;            // common residue size (0 if mixed)
    BatchGeom G{};
    std::vector<ChainDev> chains;
    std::vector<int> order, cta_start;
    cudaStream_t stream = nullptr;
    ChainDev* d_chains = nullptr;
    ChainState* d_state = nullptr;
    int* d_order = nullptr;       // chains of each CTA, CTA after CTA (d_cta_start: CSR offsets)
    int* d_cta_start = nullptr;
    int ncta = 0;
    ulonglong4_32a* d_M = nullptr;
    uint4 *d_F = nullptr, *d_FB = nullptr;
    uint16_t* d_LST = nullptr;
    int *d_NL = nullptr, *d_gorder = nullptr, *d_gcell = nullptr, *d_gstarts = nullptr, *d_res_chain = nullptr;
    uint4* d_gpos = nullptr;      // first-atom positions in cell order, w = residue (list builds)
    int *d_item_chain = nullptr, *d_chain_item0 = nullptr, *d_build = nullptr;
    int nitems = 0;               // list-build work items (home cells, or 32-residue chunks) of all chains
    double* d_prm = nullptr;
    int* d_tile_chain = nullptr;
    int* d_tile_first = nullptr;
    double* d_part = nullptr;
    int ntiles = 0;
    CutDev cut64{};
    cudaGraphExec_t graph = nullptr;
    cudaGraphExec_t tgraph = nullptr;   // the same sweep with event records around its two phases
    cudaEvent_t tev[3] = {nullptr, nullptr, nullptr};
    std::vector<double> cost;     // LPT cost of each chain's sweep
    std::vector<int> kgeom, kheur; // speculation: geometric maximum and the box-size heuristic per chain
    std::vector<char> clustered;   // chains run by a cluster of two CTAs
    int nsm = 152, ctas_per_sm = 1, spec_cap = 0, clusters = 0;
    int ncl = 0;                   // clusters (one chain each)
    int* d_cl_order = nullptr;     // their chains
    int* d_cl_start = nullptr;
    cudaStream_t stream2 = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    std::string signature;        // workload + device key of the autotuner cache
    double* d_xyz = nullptr;      // staging for host-buffer runs (3 x natoms)
    MoveLogDev* d_mlog = nullptr; // per-move records the next direct sweep launch writes (null: none)
    MoveLogDev* d_log = nullptr;  // their buffer (one record per residue of all chains), on first use
    double* d_eres = nullptr;     // per-residue energy shares (mixed recompute)
    int* d_changed = nullptr;     // chains whose coordinates the last host import changed
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    int threads = 256;
    int64_t rebuilds_seen = 0, launches = 0;
    ~mcg_batch() {
        if (graph) cudaGraphExecDestroy(graph);
        if (tgraph) cudaGraphExecDestroy(tgraph);
        for (cudaEvent_t e : tev) if (e) cudaEventDestroy(e);
        if (ev_fork) cudaEventDestroy(ev_fork);
        if (ev_join) cudaEventDestroy(ev_join);
        if (stream2) cudaStreamDestroy(stream2);
        if (d_cl_order) cudaFree(d_cl_order);
        if (d_cl_start) cudaFree(d_cl_start);
        void* p[] = {d_chains, d_state, d_order, d_M, d_F, d_FB, d_LST, d_NL, d_gorder, d_gcell, d_prm, d_tile_chain,
                     d_tile_first, d_part, d_xyz, d_gstarts, d_res_chain, d_eres, d_cta_start, d_gpos, d_item_chain,
                     d_chain_item0, d_build, d_log, d_changed};
        for (void* q : p) if (q) cudaFree(q);
        if (ev0) cudaEventDestroy(ev0);
        if (ev1) cudaEventDestroy(ev1);
        if (stream) cudaStreamDestroy(stream);
    }
    // list build: per-chain binning (every chain when force, else the chains that moved enough),
    // then one warp per home cell of the binned chains over the GPU
    int launch_build(cudaStream_t st, int force) {
        k_batch_bin<<<nchains, 1024, 0, st>>>(d_chains, d_F, d_FB, d_gstarts, d_gorder, d_gcell, d_gpos, d_state, d_build,
                                             G.pre2, force, nchains);
        const int blocks = (int)std::min<int64_t>((nitems + 7) / 8, 152 * 16);
        if (apr_all == 3)
            k_batch_lists<3><<<blocks, 256, 0, st>>>(d_chains, G, d_F, d_item_chain, d_chain_item0, d_gstarts, d_gorder, d_gpos,
                                                     d_LST, d_NL, d_state, d_build, nitems);
        else if (apr_all == 1)
            k_batch_lists<1><<<blocks, 256, 0, st>>>(d_chains, G, d_F, d_item_chain, d_chain_item0, d_gstarts, d_gorder, d_gpos,
                                                     d_LST, d_NL, d_state, d_build, nitems);
        else
            k_batch_lists<0><<<blocks, 256, 0, st>>>(d_chains, G, d_F, d_item_chain, d_chain_item0, d_gstarts, d_gorder, d_gpos,
                                                     d_LST, d_NL, d_state, d_build, nitems);
        BK(cudaGetLastError());
        launches += 2;
        return MCG_OK;
    }
    int launch_build() { return launch_build(stream, 1); }
    // slices of 256 atoms per chain for the per-atom host-buffer kernels: enough for the largest
    // chain to take about 8 atoms per thread
    int atom_slices() const {
        int mx = 1;
        for (const ChainDev& C : chains) mx = std::max(mx, C.nres * C.apr);
        return std::max(1, std::min(64, (mx + 8 * 256 - 1) / (8 * 256)));
    }
    // mixed recompute of the running energies: every chain, or the chains flagged in `only`
    // (only[nchains] != 0 when any is: the kernels return at once when none is)
    int launch_energy_list(const int* only = nullptr) {
        const int* any = only ? only + nchains : nullptr;
        int r;
        if (!d_eres && (r = balloc_d(&d_eres, (size_t)nres))) return r;
        const int blocks = (int)std::min<int64_t>((nres + 7) / 8, 152 * 16);
        if (apr_all == 3)
            k_batch_energy_res<3><<<blocks, 256, 0, stream>>>(d_chains, G, d_F, d_res_chain, d_LST, d_NL, d_eres, nres, only,
                                                              any);
        else if (apr_all == 1)
            k_batch_energy_res<1><<<blocks, 256, 0, stream>>>(d_chains, G, d_F, d_res_chain, d_LST, d_NL, d_eres, nres, only,
                                                              any);
        else
            k_batch_energy_res<0><<<blocks, 256, 0, stream>>>(d_chains, G, d_F, d_res_chain, d_LST, d_NL, d_eres, nres, only,
                                                              any);
        k_batch_energy_sum<<<nchains, 256, 0, stream>>>(d_chains, d_eres, d_state, nchains, only, any);
        BK(cudaGetLastError());
        launches += 2;
        return MCG_OK;
    }
    // One sweep as a CUDA graph: [bin, lists, sweep].  The timed variant records an event before,
    // between and after the two phases (event-record nodes) so each phase can be timed per launch.
    int capture(cudaGraphExec_t* out, bool timed) {
        const int64_t l0 = launches;
        BK(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
        cudaError_t er = cudaSuccess;
        if (timed) er = cudaEventRecordWithFlags(tev[0], stream, cudaEventRecordExternal);
        int r = er == cudaSuccess ? launch_build(stream, 0) : MCG_ECUDA;
        if (!r && timed) er = cudaEventRecordWithFlags(tev[1], stream, cudaEventRecordExternal);
        if (!r && er == cudaSuccess) r = launch_sweep(stream);
        if (!r && timed) er = cudaEventRecordWithFlags(tev[2], stream, cudaEventRecordExternal);
        cudaGraph_t g = nullptr;
        cudaError_t ee = cudaStreamEndCapture(stream, &g);
        launches = l0;            // capturing launches nothing; replays are counted per sweep
        if (r || er != cudaSuccess) {
            if (g) cudaGraphDestroy(g);
            return r ? r : fail(MCG_ECUDA, std::string("event record in capture: ") + cudaGetErrorString(er));
        }
        if (ee != cudaSuccess) return fail(MCG_ECUDA, std::string("graph capture: ") + cudaGetErrorString(ee));
        cudaError_t ie = cudaGraphInstantiate(out, g, 0);
        cudaGraphDestroy(g);
        if (ie != cudaSuccess) return fail(MCG_ECUDA, std::string("graph instantiate: ") + cudaGetErrorString(ie));
        return MCG_OK;
    }
    int ensure_graph() { return graph ? MCG_OK : capture(&graph, false); }
    // kernels one replay of the sweep graph launches: bin, lists, and the one-CTA and/or cluster sweep
    int kernels_per_sweep() const { return 2 + (ncta > 0 ? 1 : 0) + (ncl > 0 ? 1 : 0); }
    int ensure_timed_graph() {
        if (tgraph) return MCG_OK;
        for (cudaEvent_t& e : tev)
            if (!e) BK(cudaEventCreate(&e));
        return capture(&tgraph, true);
    }
    void drop_graphs() {
        if (graph) cudaGraphExecDestroy(graph);
        if (tgraph) cudaGraphExecDestroy(tgraph);
        graph = tgraph = nullptr;
    }
    // Longest-processing-time packing of chains onto ctas_per_sm persistent CTAs per SM: the cost
    // of a chain's sweep is its move count times the pairs one move touches.  The largest chains
    // get a CTA, and so an SM, of their own; smaller ones fill the least-loaded CTAs.
    // With clusters on (their CTAs have 512 threads), the largest chains whose sweep would outlast the average
    // SM load get a cluster of two CTAs (two SMs) each; the others are packed onto the remaining
    // persistent CTAs.
    int pack(int per_sm, int cl) {
        std::vector<int> idx(nchains);
        std::iota(idx.begin(), idx.end(), 0);
        std::stable_sort(idx.begin(), idx.end(), [&](int a, int b) { return cost[a] > cost[b]; });
        clustered.assign(nchains, 0);
        std::vector<int> cl_chains;
        if (cl) {
            double reg = 0.0, clc = 0.0;
            for (double v : cost) reg += v;
            for (int c : idx) {
                // a two-SM chain runs ~1.6x faster at ~1.25x the SM time
                const double avg = (reg + 1.25 * clc) / nsm;
                if (!(cost[c] > 1.1 * avg) || kgeom[c] < 2 || 2 * ((int)cl_chains.size() + 1) > nsm / 2) break;
                clustered[c] = 1;
                cl_chains.push_back(c);
                reg -= cost[c];
                clc += cost[c];
            }
        }
        ncl = (int)cl_chains.size();
        clusters = cl;
        const int nreg = nchains - ncl;
        // per_sm CTAs per SM less the cluster CTAs: with per_sm above the CTAs an SM holds, the
        // extra CTAs start as others finish (dynamic balancing of the longest-first packing)
        ncta = nreg ? std::min(nreg, std::max(1, nsm * std::max(1, per_sm) - 2 * ncl)) : 0;
        std::vector<double> load(std::max(1, ncta), 0.0);
        std::vector<std::vector<int>> per(std::max(1, ncta));
        for (int c : idx) {
            if (clustered[c]) continue;
            int best = 0;
            for (int k = 1; k < ncta; k++) if (load[k] < load[best]) best = k;
            load[best] += cost[c];
            per[best].push_back(c);
        }
        order.clear();
        cta_start.assign(ncta + 1, 0);
        for (int k = 0; k < ncta; k++) {
            cta_start[k] = (int)order.size();
            order.insert(order.end(), per[k].begin(), per[k].end());
        }
        cta_start[ncta] = (int)order.size();
        ctas_per_sm = per_sm;
        if (!d_order) {
            cudaError_t e = cudaMalloc((void**)&d_order, sizeof(int) * nchains);
            if (e != cudaSuccess) return fail(MCG_ECUDA, std::string("cudaMalloc: ") + cudaGetErrorString(e));
        }
        if (d_cta_start) { cudaFree(d_cta_start); d_cta_start = nullptr; }
        cudaError_t e = cudaMalloc((void**)&d_cta_start, sizeof(int) * (ncta + 1));
        if (e != cudaSuccess) return fail(MCG_ECUDA, std::string("cudaMalloc: ") + cudaGetErrorString(e));
        if (!order.empty())
            BK(cudaMemcpyAsync(d_order, order.data(), sizeof(int) * order.size(), cudaMemcpyHostToDevice, stream));
        BK(cudaMemcpyAsync(d_cta_start, cta_start.data(), sizeof(int) * (ncta + 1), cudaMemcpyHostToDevice, stream));
        if (ncl) {
            std::vector<int> st(ncl + 1);
            std::iota(st.begin(), st.end(), 0);
            if (d_cl_order) { cudaFree(d_cl_order); d_cl_order = nullptr; }
            if (d_cl_start) { cudaFree(d_cl_start); d_cl_start = nullptr; }
            if (cudaMalloc((void**)&d_cl_order, sizeof(int) * ncl) != cudaSuccess ||
                cudaMalloc((void**)&d_cl_start, sizeof(int) * (ncl + 1)) != cudaSuccess)
                return fail(MCG_ECUDA, "cudaMalloc of the cluster packing");
            BK(cudaMemcpyAsync(d_cl_order, cl_chains.data(), sizeof(int) * ncl, cudaMemcpyHostToDevice, stream));
            BK(cudaMemcpyAsync(d_cl_start, st.data(), sizeof(int) * (ncl + 1), cudaMemcpyHostToDevice, stream));
            if (!stream2) BK(cudaStreamCreateWithFlags(&stream2, cudaStreamNonBlocking));
            if (!ev_fork) { BK(cudaEventCreateWithFlags(&ev_fork, cudaEventDisableTiming)); BK(cudaEventCreateWithFlags(&ev_join, cudaEventDisableTiming)); }
        }
        return MCG_OK;
    }
    // Speculation width of every chain: the box-size heuristic (cap 0) or min(cap, geometric limit).
    void set_speculation(int cap) {
        for (int c = 0; c < nchains; c++) {
            const int cl = (c < (int)clustered.size() && clustered[c]) ? 2 : 1;
            int k = cap <= 0 ? kheur[c] : std::min(cap, kgeom[c]);
            // a group is whole warps, and one warp holds the atoms of all moves of an iteration
            // a group is whole warps; the kernel for residues of more than 4 atoms holds 8 records
            const int kcap = (apr_all == 1 || apr_all == 3) ? KMAX : 8;
            while (k > 1 && (k > cl * threads / 32 || k > kcap)) k >>= 1;
            chains[c].kspec = std::max(k, cl);
        }
        spec_cap = cap;
    }
    // Launch shape of the sweep; takes effect at the next sweep (the graphs are captured again).
    int reconfigure(int nthreads, int per_sm, int spec, int cl) {
        BK(cudaStreamSynchronize(stream));
        threads = nthreads;
        int r = pack(per_sm, cl);
        if (r) return r;
        set_speculation(spec);
        BK(cudaMemcpyAsync(d_chains, chains.data(), sizeof(ChainDev) * nchains, cudaMemcpyHostToDevice, stream));
        BK(cudaStreamSynchronize(stream));
        drop_graphs();
        return MCG_OK;
    }
    template <int APR>
    void sweep_kernel(cudaStream_t st) {
        if (!ncta) return;
        if (threads == 512)
            k_batch_sweep<APR, 512, 1><<<ncta, 512, 0, st>>>(d_chains, G, d_M, d_F, d_FB, d_LST, d_NL, d_gorder, d_gcell,
                                                             d_gpos, d_state, d_cta_start, d_order, nchains, d_mlog);
        else if (threads == 128)
            k_batch_sweep<APR, 128, 1><<<ncta, 128, 0, st>>>(d_chains, G, d_M, d_F, d_FB, d_LST, d_NL, d_gorder, d_gcell,
                                                             d_gpos, d_state, d_cta_start, d_order, nchains, d_mlog);
        else
            k_batch_sweep<APR, 256, 1><<<ncta, 256, 0, st>>>(d_chains, G, d_M, d_F, d_FB, d_LST, d_NL, d_gorder, d_gcell,
                                                             d_gpos, d_state, d_cta_start, d_order, nchains, d_mlog);
    }
    template <int APR>
    cudaError_t cluster_kernel(cudaStream_t st) {
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3(2 * ncl);
        cfg.blockDim = dim3(512);
        cfg.dynamicSmemBytes = 0;
        cfg.stream = st;
        cudaLaunchAttribute attr[1];
        attr[0].id = cudaLaunchAttributeClusterDimension;
        attr[0].val.clusterDim.x = 2;
        attr[0].val.clusterDim.y = 1;
        attr[0].val.clusterDim.z = 1;
        cfg.attrs = attr;
        cfg.numAttrs = 1;
        return cudaLaunchKernelEx(&cfg, k_batch_sweep<APR, 512, 2>, (const ChainDev*)d_chains, G, d_M, d_F, d_FB, d_LST,
                                  d_NL, d_gorder, d_gcell, d_gpos, d_state, (const int*)d_cl_start, (const int*)d_cl_order,
                                  nchains, d_mlog);
    }
    // The cluster chains on a second stream branch, concurrently with the regular CTAs.
    int launch_sweep(cudaStream_t st) {
        if (ncl) {
            BK(cudaEventRecord(ev_fork, st));
            BK(cudaStreamWaitEvent(stream2, ev_fork, 0));
            if (apr_all == 3) BK(cluster_kernel<3>(stream2));
            else if (apr_all == 1) BK(cluster_kernel<1>(stream2));
            else BK(cluster_kernel<0>(stream2));
            BK(cudaEventRecord(ev_join, stream2));
        }
        if (apr_all == 3) sweep_kernel<3>(st);
        else if (apr_all == 1) sweep_kernel<1>(st);
        else sweep_kernel<0>(st);
        BK(cudaGetLastError());
        if (ncl) BK(cudaStreamWaitEvent(st, ev_join, 0));
        return MCG_OK;
    }
};

template <typename T>
static int balloc(T** p, size_t n) {
    cudaError_t e = cudaMalloc((void**)p, std::max<size_t>(1, n) * sizeof(T));
    if (e != cudaSuccess) return fail(MCG_ECUDA, std::string("cudaMalloc: ") + cudaGetErrorString(e));
    return MCG_OK;
}

extern "C" {

int mcg_batch_create(const mcg_system_desc* descs, int nchains, const mcg_batch_opts* opts, mcg_batch** out) {
    if (!out) return fail(MCG_EINVAL, "null output handle");
    *out = nullptr;
    if (!descs || nchains <= 0 || !opts) return fail(MCG_EINVAL, "need chains and options");
    if (!(opts->dmax_trn >= 0) || !(opts->dmax_rot >= 0)) return fail(MCG_EINVAL, "dmax values must be >= 0");
    // dmax adjustment: periods, targets and the caps the sweep's geometry is sized for
    double dmax_cap[2];
    {
        const double init[2] = {opts->dmax_trn, opts->dmax_rot};
        for (int t = 0; t < 2; t++) {
            if (opts->dmax_each[t] < 0) return fail(MCG_EINVAL, "dmax_each must be >= 0");
            if (!(opts->dmax_target[t] >= 0.0 && opts->dmax_target[t] <= 100.0))
                return fail(MCG_EINVAL, "dmax_target must be a percentage in [0, 100]");
            if (!(opts->dmax_max[t] >= 0.0)) return fail(MCG_EINVAL, "dmax_max must be >= 0");
            dmax_cap[t] = opts->dmax_max[t] > 0.0 ? opts->dmax_max[t] : (opts->dmax_each[t] > 0 ? 2.0 * init[t] : init[t]);
            if (dmax_cap[t] < init[t]) return fail(MCG_EINVAL, "dmax_max is below the initial dmax");
        }
        if (dmax_cap[1] > 180.0) return fail(MCG_EINVAL, "the rotation dmax cap exceeds 180 degrees");
    }
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= 0) { cudaGetLastError(); return fail(MCG_ECUDA, "no CUDA device available"); }
    std::unique_ptr<mcg_batch> B(new mcg_batch);
    B->nchains = nchains;
    const mcg_system_desc& d0 = descs[0];
    const double rc = d0.cutoff, ron = d0.cuton, skin = d0.dcut > 0 ? d0.dcut : 2.0;
    std::vector<ulonglong4_32a> M;
    std::vector<uint4> F;
    std::vector<double> prm;
    double rext = 0.0;       // largest distance from a residue's first atom to its other atoms
    double span_max = 0.0;   // largest intra-residue distance
    int apr_all = -1;
    int64_t atom0 = 0, res0 = 0;
    B->chains.resize(nchains);
    for (int c = 0; c < nchains; c++) {
        const mcg_system_desc& d = descs[c];
        HostSystem hs;
        int rc2 = build_host_system(&d, hs);
        if (rc2) return fail(rc2, "chain " + std::to_string(c) + ": " + mcg_last_error());
        if (hs.cut != MCG_CUT_SWITCH) return fail(MCG_EINVAL, "batched chains need the switch cutoff");
        if (hs.pbc == MCG_PBC_NONE) return fail(MCG_EINVAL, "batched chains need periodic boxes");
        if (d.cutoff != rc || d.cuton != ron || d.dcut != d0.dcut) return fail(MCG_EINVAL, "all chains must share cutoff, cuton and skin");
        if (!hs.pairs14.empty()) return fail(MCG_ENOTSUP, "batched chains hold rigid residues without 1-4 pairs");
        for (int i = 0; i < hs.n; i++) if (hs.frozen[i]) return fail(MCG_ENOTSUP, "frozen atoms are not supported in batched chains");
        int apr = 0;
        while (apr < hs.n && hs.resid[apr] == hs.resid[0]) apr++;
        if (apr < 1 || apr > MAX_APR || hs.n % apr) return fail(MCG_ENOTSUP, "residues must all have the same size (1..8 atoms)");
        const int nres = hs.n / apr;
        if (nres > 65535) return fail(MCG_ENOTSUP, "at most 65535 residues per chain");
        for (int r = 0; r < nres; r++)
            for (int k = 0; k < apr; k++) {
                int a = r * apr + k;
                if (hs.resid[a] != hs.resid[r * apr] || (r > 0 && hs.resid[a] == hs.resid[a - apr]))
                    return fail(MCG_ENOTSUP, "residues must all have the same size");
                if (hs.q[a] != hs.q[k] || hs.eps[a] != hs.eps[k] || hs.sig[a] != hs.sig[k])
                    return fail(MCG_ENOTSUP, "residues must share one parameter template");
                for (int k2 = k + 1; k2 < apr; k2++) {
                    int b = r * apr + k2;
                    bool ex = false;
                    for (int t = hs.exclStart[a]; t < hs.exclStart[a + 1]; t++) ex |= hs.exclData[t] == b;
                    if (!ex) return fail(MCG_ENOTSUP, "every intra-residue pair must be excluded (rigid residues)");
                }
            }
        if (apr_all < 0) apr_all = apr; else if (apr_all != apr) apr_all = 0;
        ChainDev& C = B->chains[c];
        memset(&C, 0, sizeof C);
        C.atom0 = (int)atom0; C.res0 = (int)res0; C.nres = nres; C.apr = apr;
        for (int k = 0; k < 3; k++) {
            C.L[k] = hs.L[k]; C.rL[k] = hs.rL[k];
            C.tofix32[k] = (float)(4294967296.0 / hs.L[k]);
            C.Ls[k] = (float)(hs.L[k] / 4294967296.0);
            C.Lsl[k] = (float)(hs.L[k] / 4294967296.0 - (double)C.Ls[k]);
        }
        C.beta = 1.0 / ((RBOLTZUI / KCALTOIU) * hs.temp);
        if (opts->acceptance_units == MCG_ACCEPT_PHYSICAL) C.beta /= KCALTOIU;
        C.beta_f = (float)C.beta;
        C.dmax_trn = (float)opts->dmax_trn;
        C.dmax_rot = (float)opts->dmax_rot;
        for (int t = 0; t < 2; t++) {
            C.each[t] = opts->dmax_each[t];
            C.target[t] = opts->dmax_target[t] / 100.0;
            C.dmax_cap[t] = dmax_cap[t];
        }
        C.ntypes_move = apr > 1 ? 2 : 1;
        uint64_t key = (opts->seed + 1) * 0x9E3779B97F4A7C15ull ^ ((uint64_t)c * 0xD1B54A32D192ED03ull);
        C.key0 = (uint32_t)key; C.key1 = (uint32_t)(key >> 32);
        const double K = CHGCHARMM * KCALTOIU;
        for (int a = 0; a < apr; a++)
            for (int b = 0; b < apr; b++) {
                const double qk = K * hs.q[a] * hs.q[b];
                C.tab[a][b][0] = (float)qk;
                C.tab[a][b][3] = (float)(qk - (double)(float)qk);
                const double e4 = 4.0 * hs.eps[a] * hs.eps[b];
                C.tab[a][b][1] = (float)e4;
                C.tablo[a][b][0] = (float)(e4 - (double)(float)e4);
                double s = hs.sig[a] + hs.sig[b];
                C.tab[a][b][2] = (float)(s * s);
                C.tablo[a][b][1] = (float)(s * s - (double)(float)(s * s));
            }
        for (int i = 0; i < hs.n; i++) {
            ulonglong4_32a m;
            m.x = host_master(hs.x[i], hs.rL[0]); m.y = host_master(hs.y[i], hs.rL[1]); m.z = host_master(hs.z[i], hs.rL[2]); m.w = 0;
            M.push_back(m);
            F.push_back(make_uint4((uint32_t)(m.x >> 32), (uint32_t)(m.y >> 32), (uint32_t)(m.z >> 32), (uint32_t)(i % apr)));
            prm.push_back(hs.q[i]); prm.push_back(hs.eps[i]); prm.push_back(hs.sig[i]);
        }
        for (int r = 0; r < nres; r++)
            for (int k = 0; k < apr; k++)
                for (int k2 = k + 1; k2 < apr; k2++) {
                    const int i = r * apr + k, j = r * apr + k2;
                    double e[3] = {hs.x[j] - hs.x[i], hs.y[j] - hs.y[i], hs.z[j] - hs.z[i]};
                    for (int t = 0; t < 3; t++) e[t] -= hs.L[t] * std::nearbyint(e[t] * hs.rL[t]);
                    const double d = std::sqrt(e[0] * e[0] + e[1] * e[1] + e[2] * e[2]);
                    span_max = std::max(span_max, d);
                    if (k == 0) rext = std::max(rext, d);
                }
        atom0 += hs.n;
        res0 += nres;
        if (atom0 > (int64_t)2000000000) return fail(MCG_EINVAL, "too many atoms");
    }
    B->natoms = atom0;
    B->nres = res0;
    B->apr_all = apr_all;
    BatchGeom& G = B->G;
    G.c2f = (float)(rc * rc); G.n2f = (float)(ron * ron);
    { double dd = rc * rc - ron * ron; G.sw2f = (float)(1.0 / (dd * dd * dd)); }
    const double rlist = rc + skin;
    G.rlist2 = (float)(rlist * rlist);
    rext += 0.01;
    G.rcent2 = (float)((rlist + 2 * rext) * (rlist + 2 * rext));
    G.half_skin2 = (float)(0.25 * skin * skin);
    G.cellmin = (float)(0.5 * (rlist + 2 * rext) + 1e-3);
    // dE forms the new displacement as d_old - m; that is the minimum image for every pair inside
    // the cutoff only while rc + |m| <= L/2 (m: the largest move of one atom)
    const double span = span_max + 0.01;   // rigid residues keep their intra-residue distances
    const double mmax = std::max(dmax_cap[0], 2.0 * span * std::sin(0.5 * dmax_cap[1] * PI / 180.0)) + 1e-6;
    const double rind = rc + 2.0 * rext + 2.0 * mmax + 1e-3;
    G.indep2 = (float)(rind * rind);
    // pre-sweep rebuild threshold: lower rebuilds more chains before each sweep, higher leaves more
    // rebuilds to the chains' own CTAs inside the sweep; on the 256-chain water workload (steady
    // state) 0.55, 0.75, 0.9 and 1.0 half-skins took 15.1, 14.7, 16.7 and 17.1 ms per sweep
    G.pre2 = (float)((0.7 * 0.5 * skin) * (0.7 * 0.5 * skin));
    G.pair2 = (float)((rc + 2.0 * rext + 1e-3) * (rc + 2.0 * rext + 1e-3));
    {
        const double rs = rlist + 2 * rext + skin + 0.01;
        G.subst2 = (float)(rs * rs);
    }
    for (auto& C : B->chains) {
        for (int k = 0; k < 3; k++) {
            if (rc + mmax > 0.5 * C.L[k])
                return fail(MCG_EINVAL, "cutoff plus the largest move exceeds half a chain's box");
            C.nc[k] = (int)std::floor(C.L[k] / G.cellmin);
        }
        C.use_cells = (C.nc[0] >= 5 && C.nc[1] >= 5 && C.nc[2] >= 5 && C.nc[0] * C.nc[1] * C.nc[2] <= MAX_CELLS) ? 1 : 0;
        for (int k = 0; k < 3; k++) { C.Lf[k] = (float)C.L[k]; C.Lhalf[k] = (float)(0.5 * C.L[k]); }
        C.wrap_offsets = (rc + rext + mmax + span > 0.5 * std::min(C.L[0], std::min(C.L[1], C.L[2]))) ? 1 : 0;
        // speculation width: a move is re-proposed only when an earlier accepted move of its
        // iteration picked the same residue (interacting moves are corrected, not re-proposed);
        // take the widest group in which that happens in under ~5% of the iterations (~0.5
        // acceptance assumed): 8 from 140 residues, 16 from 1,200, 32 (two-CTA clusters) from 4,960
        {
            int kh = 1;
            for (int kw : {2, 4, 8, 16, 32})
                if (0.5 * 0.5 * kw * (kw - 1) / (double)C.nres <= 0.05) kh = kw;
            B->kgeom.push_back(KMAX);
            B->kheur.push_back(kh);
        }
        if (!C.use_cells) C.nc[0] = C.nc[1] = C.nc[2] = 1;
    }
    if (opts->list_capacity > 0) G.cap = opts->list_capacity;
    else {
        double dens = 0;
        int maxres = 0;
        for (auto& C : B->chains) { dens = std::max(dens, C.nres / (C.L[0] * C.L[1] * C.L[2])); maxres = std::max(maxres, C.nres); }
        double r = rlist + 2 * rext;
        G.cap = (int)(4.0 / 3.0 * PI * r * r * r * dens * 1.6) + 64;
        G.cap = std::min((G.cap + 31) & ~31, ((maxres + 31) & ~31) + 32);
    }
    if (G.cap > 65535) G.cap = 65535;
    B->threads = opts->threads_per_chain > 0 ? opts->threads_per_chain : 512;
    if (B->threads != 128 && B->threads != 256 && B->threads != 512)
        return fail(MCG_EINVAL, "threads_per_chain must be 128, 256 or 512");
    if (opts->speculation < 0 || (opts->speculation & (opts->speculation - 1)) || opts->speculation > KMAX)
        return fail(MCG_EINVAL, "speculation must be 0, 1, 2, 4, 8, 16 or 32");
    if (opts->ctas_per_sm < 0 || opts->ctas_per_sm > 8) return fail(MCG_EINVAL, "ctas_per_sm must be in [0, 8]");
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&B->nsm, cudaDevAttrMultiProcessorCount, dev);
    B->cost.resize(nchains);
    {
        const double rl = rc + skin;
        uint64_t h = 1469598103934665603ull;       // FNV-1a over the workload's shape
        auto mix = [&](uint64_t v) { for (int k = 0; k < 8; k++) { h ^= (v >> (8 * k)) & 0xff; h *= 1099511628211ull; } };
        for (int c = 0; c < nchains; c++) {
            const ChainDev& C = B->chains[c];
            const double dens = C.nres / (C.L[0] * C.L[1] * C.L[2]);
            const double neigh = std::min((double)C.nres, dens * 4.0 / 3.0 * PI * rl * rl * rl);
            B->cost[c] = (double)C.nres * neigh * C.apr * C.apr + 1.0;
            mix((uint64_t)C.nres); mix((uint64_t)C.apr); mix((uint64_t)llround(C.L[0] * 1000));
        }
        mix((uint64_t)llround(rc * 1000)); mix((uint64_t)llround(skin * 1000));
        mix((uint64_t)llround(opts->dmax_trn * 1e4)); mix((uint64_t)llround(opts->dmax_rot * 1e4));
        for (int t = 0; t < 2; t++) {
            mix((uint64_t)opts->dmax_each[t]); mix((uint64_t)llround(opts->dmax_target[t] * 1e4));
            mix((uint64_t)llround(dmax_cap[t] * 1e4));
        }
        cudaDeviceProp prop;
        std::string name = cudaGetDeviceProperties(&prop, dev) == cudaSuccess ? prop.name : "unknown";
        for (char& ch : name) if (ch == ' ') ch = '_';
        char buf[64];
        snprintf(buf, sizeof buf, "%016llx", (unsigned long long)h);
        B->signature = name + ":" + std::to_string(nchains) + ":" + buf;
    }
    BK(cudaStreamCreateWithFlags(&B->stream, cudaStreamNonBlocking));
    int r;
    if (opts->clusters < -1 || opts->clusters > 1) return fail(MCG_EINVAL, "clusters must be -1, 0 or 1");
    if ((r = B->pack(opts->ctas_per_sm > 0 ? opts->ctas_per_sm : 1, opts->clusters >= 0 ? 1 : 0))) return r;
    B->set_speculation(opts->speculation);
    if ((r = balloc(&B->d_chains, nchains)) || (r = balloc(&B->d_state, nchains)) ||
        (r = balloc(&B->d_M, atom0)) || (r = balloc(&B->d_F, atom0)) || (r = balloc(&B->d_FB, atom0)) ||
        (r = balloc(&B->d_LST, (size_t)res0 * G.cap)) || (r = balloc(&B->d_NL, res0)) || (r = balloc(&B->d_gorder, res0)) ||
        (r = balloc(&B->d_gcell, res0)) || (r = balloc(&B->d_prm, prm.size())) ||
        (r = balloc(&B->d_gstarts, (size_t)nchains * (MAX_CELLS + 1))) || (r = balloc(&B->d_res_chain, res0)) ||
        (r = balloc(&B->d_gpos, res0)))
        return r;
    {
        std::vector<int> rcn(res0);
        for (int c = 0; c < nchains; c++)
            for (int k = 0; k < B->chains[c].nres; k++) rcn[B->chains[c].res0 + k] = c;
        BK(cudaMemcpy(B->d_res_chain, rcn.data(), sizeof(int) * res0, cudaMemcpyHostToDevice));
    }
    BK(cudaMemcpyAsync(B->d_chains, B->chains.data(), sizeof(ChainDev) * nchains, cudaMemcpyHostToDevice, B->stream));
    BK(cudaMemcpyAsync(B->d_M, M.data(), sizeof(ulonglong4_32a) * atom0, cudaMemcpyHostToDevice, B->stream));
    BK(cudaMemcpyAsync(B->d_F, F.data(), sizeof(uint4) * atom0, cudaMemcpyHostToDevice, B->stream));
    BK(cudaMemcpyAsync(B->d_prm, prm.data(), sizeof(double) * prm.size(), cudaMemcpyHostToDevice, B->stream));
    BK(cudaMemsetAsync(B->d_state, 0, sizeof(ChainState) * nchains, B->stream));
    std::vector<int> tc, tf;
    for (int c = 0; c < nchains; c++) {
        int n = B->chains[c].nres * B->chains[c].apr;
        for (int f = 0; f < n; f += ETILE) { tc.push_back(c); tf.push_back(f); }
    }
    B->ntiles = (int)tc.size();
    if ((r = balloc(&B->d_tile_chain, tc.size())) || (r = balloc(&B->d_tile_first, tf.size())) || (r = balloc(&B->d_part, tc.size())))
        return r;
    BK(cudaMemcpyAsync(B->d_tile_chain, tc.data(), sizeof(int) * tc.size(), cudaMemcpyHostToDevice, B->stream));
    {
        std::vector<int> ic, i0(nchains);
        for (int c = 0; c < nchains; c++) {
            const ChainDev& C = B->chains[c];
            const int n = C.use_cells ? C.nc[0] * C.nc[1] * C.nc[2] : (C.nres + 31) / 32;
            i0[c] = (int)ic.size();
            ic.insert(ic.end(), n, c);
        }
        B->nitems = (int)ic.size();
        if ((r = balloc(&B->d_item_chain, ic.size())) || (r = balloc(&B->d_chain_item0, nchains)) || (r = balloc(&B->d_build, nchains)))
            return r;
        BK(cudaMemcpy(B->d_item_chain, ic.data(), sizeof(int) * ic.size(), cudaMemcpyHostToDevice));
        BK(cudaMemcpy(B->d_chain_item0, i0.data(), sizeof(int) * nchains, cudaMemcpyHostToDevice));
    }
    BK(cudaMemcpyAsync(B->d_tile_first, tf.data(), sizeof(int) * tf.size(), cudaMemcpyHostToDevice, B->stream));
    B->cut64.mode = 1;
    B->cut64.c2 = rc * rc; B->cut64.n2 = ron * ron;
    { double dd = B->cut64.c2 - B->cut64.n2; B->cut64.sw2 = 1. / (dd * dd * dd); }
    if ((r = B->launch_build())) return r;
    std::vector<double> e(nchains);
    r = mcg_batch_energy_fp64(B.get(), e.data());
    if (r) return r;
    std::vector<ChainState> st(nchains);
    BK(cudaMemcpyAsync(st.data(), B->d_state, sizeof(ChainState) * nchains, cudaMemcpyDeviceToHost, B->stream));
    BK(cudaStreamSynchronize(B->stream));
    for (int c = 0; c < nchains; c++) {
        if (st[c].err) return fail(st[c].err, "neighbour list capacity exceeded (chain " + std::to_string(c) + ")");
        st[c].etot = e[c];
        st[c].dmax[0] = opts->dmax_trn;
        st[c].dmax[1] = opts->dmax_rot;
    }
    BK(cudaMemcpyAsync(B->d_state, st.data(), sizeof(ChainState) * nchains, cudaMemcpyHostToDevice, B->stream));
    BK(cudaStreamSynchronize(B->stream));
    *out = B.release();
    return MCG_OK;
}

int mcg_batch_destroy(mcg_batch* b) {
    delete b;
    return MCG_OK;
}

int mcg_batch_sweep(mcg_batch* b, int nsweeps) {
    if (!b || nsweeps < 0) return fail(MCG_EINVAL, "bad arguments");
    int r = b->ensure_graph();
    if (r) return r;
    for (int s = 0; s < nsweeps; s++) BK(cudaGraphLaunch(b->graph, b->stream));
    b->launches += b->kernels_per_sweep() * (int64_t)nsweeps;
    return MCG_OK;
}

int mcg_batch_sweep_logged(mcg_batch* b, mcg_batch_move* moves, int64_t cap) {
    if (!b || !moves) return fail(MCG_EINVAL, "null argument");
    if (cap < b->nres) return fail(MCG_EINVAL, "the record buffer needs one entry per residue of all chains");
    int r;
    if (!b->d_log && (r = balloc(&b->d_log, (size_t)b->nres))) return r;
    BK(cudaMemsetAsync(b->d_log, 0, sizeof(MoveLogDev) * b->nres, b->stream));
    // the sweep graph's kernels with the record pointer set, launched directly (the graph keeps null)
    b->d_mlog = b->d_log;
    r = b->launch_build(b->stream, 0);
    if (!r) r = b->launch_sweep(b->stream);
    b->d_mlog = nullptr;
    if (r) return r;
    b->launches += (b->ncta > 0 ? 1 : 0) + (b->ncl > 0 ? 1 : 0);
    BK(cudaMemcpyAsync(moves, b->d_log, sizeof(MoveLogDev) * b->nres, cudaMemcpyDeviceToHost, b->stream));
    BK(cudaStreamSynchronize(b->stream));
    for (const ChainDev& C : b->chains)
        for (int k = 0; k < C.nres; k++) {
            mcg_batch_move& m = moves[C.res0 + k];
            for (int j = 0; j < C.apr; j++)
                for (int t = 0; t < 3; t++) {
                    uint64_t raw;
                    std::memcpy(&raw, &m.xyz[j][t], sizeof raw);
                    m.xyz[j][t] = host_view(raw, C.L[t]);
                }
        }
    return MCG_OK;
}

int mcg_batch_time_sweeps(mcg_batch* b, int nsweeps, float* ms) {
    if (!b || nsweeps < 0 || !ms) return fail(MCG_EINVAL, "bad arguments");
    int r = b->ensure_graph();
    if (r) return r;
    if (!b->ev0) { BK(cudaEventCreate(&b->ev0)); BK(cudaEventCreate(&b->ev1)); }
    BK(cudaStreamSynchronize(b->stream));
    BK(cudaEventRecord(b->ev0, b->stream));
    for (int s = 0; s < nsweeps; s++) BK(cudaGraphLaunch(b->graph, b->stream));
    BK(cudaEventRecord(b->ev1, b->stream));
    BK(cudaEventSynchronize(b->ev1));
    BK(cudaEventElapsedTime(ms, b->ev0, b->ev1));
    b->launches += b->kernels_per_sweep() * (int64_t)nsweeps;
    return MCG_OK;
}

int mcg_batch_time_phases(mcg_batch* b, int nsweeps, float* ms_total, float* ms_lists, float* ms_sweep) {
    if (!b || nsweeps < 0 || !ms_total || !ms_lists || !ms_sweep) return fail(MCG_EINVAL, "bad arguments");
    int r = b->ensure_timed_graph();
    if (r) return r;
    if (!b->ev0) { BK(cudaEventCreate(&b->ev0)); BK(cudaEventCreate(&b->ev1)); }
    BK(cudaStreamSynchronize(b->stream));
    BK(cudaEventRecord(b->ev0, b->stream));
    double tl = 0.0, ts = 0.0;
    for (int s = 0; s < nsweeps; s++) {
        BK(cudaGraphLaunch(b->tgraph, b->stream));
        BK(cudaEventSynchronize(b->tev[2]));       // the phase events hold only the latest replay
        float a = 0.f, c = 0.f;
        BK(cudaEventElapsedTime(&a, b->tev[0], b->tev[1]));
        BK(cudaEventElapsedTime(&c, b->tev[1], b->tev[2]));
        tl += a;
        ts += c;
    }
    BK(cudaEventRecord(b->ev1, b->stream));
    BK(cudaEventSynchronize(b->ev1));
    BK(cudaEventElapsedTime(ms_total, b->ev0, b->ev1));
    *ms_lists = (float)tl;
    *ms_sweep = (float)ts;
    b->launches += b->kernels_per_sweep() * (int64_t)nsweeps;
    return MCG_OK;
}

// Autotuner cache: signature -> (threads, ctas per SM, speculation), kept for the process and,
// when MCG_TUNE_CACHE names a file, in that file (one "signature threads ctas spec ms" per line).
static std::mutex g_tune_mu;
static std::map<std::string, mcg_batch_tuning> g_tune_cache;

// A cached shape is used only if mcg_batch_create would accept it as options: a damaged or
// hand-edited cache line is skipped (and the shapes timed again), never launched.
static bool tuning_valid(const mcg_batch_tuning& v) {
    const bool th = v.threads_per_chain == 128 || v.threads_per_chain == 256 || v.threads_per_chain == 512;
    const bool cp = v.ctas_per_sm >= 1 && v.ctas_per_sm <= 8;
    const bool sp = v.speculation >= 0 && v.speculation <= KMAX && (v.speculation & (v.speculation - 1)) == 0;
    const bool cl = v.clusters == 0 || v.clusters == 1;
    return th && cp && sp && cl && std::isfinite(v.ms_per_sweep);
}

static bool tune_lookup(const std::string& sig, mcg_batch_tuning* t) {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    auto it = g_tune_cache.find(sig);
    if (it != g_tune_cache.end()) { *t = it->second; return true; }
    const char* path = getenv("MCG_TUNE_CACHE");
    if (!path || !*path) return false;
    FILE* f = fopen(path, "r");
    if (!f) return false;
    char key[256];
    mcg_batch_tuning v{};
    bool found = false;
    while (fscanf(f, "%255s %d %d %d %d %f", key, &v.threads_per_chain, &v.ctas_per_sm, &v.speculation, &v.clusters,
                  &v.ms_per_sweep) == 6)
        if (sig == key && tuning_valid(v)) { *t = v; found = true; }
    fclose(f);
    if (found) g_tune_cache[sig] = *t;
    return found;
}

static void tune_store(const std::string& sig, const mcg_batch_tuning& t) {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    g_tune_cache[sig] = t;
    const char* path = getenv("MCG_TUNE_CACHE");
    if (!path || !*path) return;
    FILE* f = fopen(path, "a");
    if (!f) return;
    fprintf(f, "%s %d %d %d %d %.4f\n", sig.c_str(), t.threads_per_chain, t.ctas_per_sm, t.speculation, t.clusters,
            t.ms_per_sweep);
    fclose(f);
}

int mcg_batch_autotune(mcg_batch* b, int trial_sweeps, int use_cache, mcg_batch_tuning* out) {
    if (!b || trial_sweeps < 1 || trial_sweeps > 64) return fail(MCG_EINVAL, "trial_sweeps must be in [1, 64]");
    mcg_batch_tuning best{};
    if (use_cache && tune_lookup(b->signature, &best)) {
        int r = b->reconfigure(best.threads_per_chain, best.ctas_per_sm, best.speculation, best.clusters);
        if (r) return r;
        best.from_cache = 1;
        if (out) *out = best;
        return MCG_OK;
    }
    // (threads per CTA, CTAs per SM): one chain per SM at 512 threads (also as two waves), two
    // co-resident chains at 256, four at 128, and eight at 128 (co-resident for one-atom residues,
    // whose kernel fits 64 registers)
    static const int kShape[][2] = {{512, 1}, {512, 2}, {256, 2}, {128, 4}, {128, 8}};
    static const int kSpec[] = {1, 2, 4, 8, 0};   // 0: the widest width the chain's size allows
    struct Cand { int th, cp, sp, cl; float ms; };
    std::vector<Cand> cand;
    if (!b->ev0) { BK(cudaEventCreate(&b->ev0)); BK(cudaEventCreate(&b->ev1)); }
    // ms per sweep of the current shape over `n` sweeps, after one warm-up sweep (graph upload)
    auto time_shape = [&](const Cand& c, int n, float* ms) -> int {
        int r = b->reconfigure(c.th, c.cp, c.sp, c.cl);
        if (r) return r;
        if ((r = b->ensure_graph())) return r;
        BK(cudaGraphLaunch(b->graph, b->stream));
        BK(cudaEventRecord(b->ev0, b->stream));
        for (int s = 0; s < n; s++) BK(cudaGraphLaunch(b->graph, b->stream));
        BK(cudaEventRecord(b->ev1, b->stream));
        BK(cudaEventSynchronize(b->ev1));
        BK(cudaEventElapsedTime(ms, b->ev0, b->ev1));
        *ms /= (float)n;
        b->launches += b->kernels_per_sweep() * (int64_t)(n + 1);
        return MCG_OK;
    };
    // stage 1: every shape
    for (const auto& shp : kShape)
        for (int sp : kSpec)
            for (int cl = 0; cl < 2; cl++) {
                Cand c{shp[0], shp[1], sp, cl, 0.f};
                int r = time_shape(c, trial_sweeps, &c.ms);
                if (r) return r;
                cand.push_back(c);
            }
    // stage 2: the six fastest again, in interleaved rounds (the chains drift while they are timed)
    std::stable_sort(cand.begin(), cand.end(), [](const Cand& x, const Cand& y) { return x.ms < y.ms; });
    cand.resize(std::min<size_t>(6, cand.size()));
    std::vector<float> sum(cand.size(), 0.f);
    for (int round = 0; round < 3; round++)
        for (size_t k = 0; k < cand.size(); k++) {
            float ms = 0.f;
            int r = time_shape(cand[k], 1, &ms);
            if (r) return r;
            sum[k] += ms;
        }
    size_t bi = 0;
    for (size_t k = 1; k < cand.size(); k++) if (sum[k] < sum[bi]) bi = k;
    best.threads_per_chain = cand[bi].th;
    best.ctas_per_sm = cand[bi].cp;
    best.speculation = cand[bi].sp;
    best.clusters = cand[bi].cl;
    best.ms_per_sweep = sum[bi] / 3.0f;
    int r = b->reconfigure(best.threads_per_chain, best.ctas_per_sm, best.speculation, best.clusters);
    if (r) return r;
    best.from_cache = 0;
    tune_store(b->signature, best);
    if (out) *out = best;
    return MCG_OK;
}

int mcg_batch_get_tuning(mcg_batch* b, mcg_batch_tuning* out) {
    if (!b || !out) return fail(MCG_EINVAL, "null argument");
    out->threads_per_chain = b->threads;
    out->ctas_per_sm = b->ctas_per_sm;
    out->speculation = b->spec_cap;
    out->clusters = b->clusters;
    out->ms_per_sweep = 0.f;
    out->from_cache = 0;
    return MCG_OK;
}

// The device address of a pinned (page-locked) host buffer, or null for any other pointer: the
// import and export kernels then read and write the host buffer themselves over the coherent
// host link, without a staging copy through device memory.
static const double* pinned_alias(const double* p) {
    cudaPointerAttributes at;
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
        cudaGetLastError();   // an unregistered pointer: not an error of this call
        return nullptr;
    }
    return at.type == cudaMemoryTypeHost ? (const double*)at.devicePointer : nullptr;
}

int mcg_batch_run_host(mcg_batch* b, const double* xyz_in, int nsweeps, double* xyz_out, int64_t* accepted, double* etot) {
    if (!b || nsweeps < 0) return fail(MCG_EINVAL, "bad arguments");
    const size_t bytes = sizeof(double) * 3 * (size_t)b->natoms;
    int r;
    const double* in_dev = xyz_in ? pinned_alias(xyz_in) : nullptr;
    double* out_dev = xyz_out ? const_cast<double*>(pinned_alias(xyz_out)) : nullptr;
    if (((xyz_in && !in_dev) || (xyz_out && !out_dev)) && !b->d_xyz) {
        if ((r = balloc(&b->d_xyz, 3 * (size_t)b->natoms))) return r;
    }
    if (xyz_in && !b->d_changed && (r = balloc(&b->d_changed, (size_t)b->nchains + 1))) return r;
    if (xyz_in) {
        if (!in_dev) {
            BK(cudaMemcpyAsync(b->d_xyz, xyz_in, bytes, cudaMemcpyHostToDevice, b->stream));
            in_dev = b->d_xyz;
        }
        BK(cudaMemsetAsync(b->d_changed, 0, sizeof(int) * ((size_t)b->nchains + 1), b->stream));
        k_batch_import<<<dim3(b->nchains, b->atom_slices()), 256, 0, b->stream>>>(b->d_chains, in_dev, b->natoms, b->d_M,
                                                                                  b->d_F, b->d_FB, b->d_state,
                                                                                  b->d_changed, b->nchains);
        BK(cudaGetLastError());
        b->launches++;
        // lists of the chains whose atoms moved beyond the rebuild threshold, then the energies of
        // the chains whose coordinates changed
        if ((r = b->launch_build(b->stream, 0)) || (r = b->launch_energy_list(b->d_changed))) return r;
    }
    if ((r = mcg_batch_sweep(b, nsweeps))) return r;
    if (xyz_out) {
        k_batch_export<<<dim3(b->nchains, b->atom_slices()), 256, 0, b->stream>>>(b->d_chains, b->d_M, b->natoms,
                                                                                  out_dev ? out_dev : b->d_xyz, b->nchains);
        BK(cudaGetLastError());
        b->launches++;
        if (!out_dev) BK(cudaMemcpyAsync(xyz_out, b->d_xyz, bytes, cudaMemcpyDeviceToHost, b->stream));
    }
    return mcg_batch_stats(b, nullptr, accepted, etot);
}

int mcg_batch_get_dmax(mcg_batch* b, double* dmax_trn, double* dmax_rot) {
    if (!b || !dmax_trn || !dmax_rot) return fail(MCG_EINVAL, "null argument");
    std::vector<ChainState> st(b->nchains);
    BK(cudaMemcpyAsync(st.data(), b->d_state, sizeof(ChainState) * b->nchains, cudaMemcpyDeviceToHost, b->stream));
    BK(cudaStreamSynchronize(b->stream));
    for (int c = 0; c < b->nchains; c++) { dmax_trn[c] = st[c].dmax[0]; dmax_rot[c] = st[c].dmax[1]; }
    return MCG_OK;
}

int mcg_batch_energy_mixed(mcg_batch* b, double* e) {
    if (!b || !e) return fail(MCG_EINVAL, "null argument");
    std::vector<ChainState> keep(b->nchains);
    BK(cudaMemcpyAsync(keep.data(), b->d_state, sizeof(ChainState) * b->nchains, cudaMemcpyDeviceToHost, b->stream));
    int r = b->launch_energy_list();
    if (r) return r;
    std::vector<ChainState> st(b->nchains);
    BK(cudaMemcpyAsync(st.data(), b->d_state, sizeof(ChainState) * b->nchains, cudaMemcpyDeviceToHost, b->stream));
    BK(cudaStreamSynchronize(b->stream));
    for (int c = 0; c < b->nchains; c++) e[c] = st[c].etot;
    BK(cudaMemcpyAsync(b->d_state, keep.data(), sizeof(ChainState) * b->nchains, cudaMemcpyHostToDevice, b->stream));
    BK(cudaStreamSynchronize(b->stream));
    return MCG_OK;
}

int mcg_batch_pairs(mcg_batch* b, int64_t* pairs) {
    if (!b || !pairs) return fail(MCG_EINVAL, "null argument");
    std::vector<ChainState> st(b->nchains);
    BK(cudaMemcpyAsync(st.data(), b->d_state, sizeof(ChainState) * b->nchains, cudaMemcpyDeviceToHost, b->stream));
    BK(cudaStreamSynchronize(b->stream));
    for (int c = 0; c < b->nchains; c++) pairs[c] = st[c].pairs;
    return MCG_OK;
}

int mcg_batch_stats(mcg_batch* b, int64_t* trials, int64_t* accepted, double* etot) {
    if (!b) return fail(MCG_EINVAL, "null handle");
    std::vector<ChainState> st(b->nchains);
    BK(cudaMemcpyAsync(st.data(), b->d_state, sizeof(ChainState) * b->nchains, cudaMemcpyDeviceToHost, b->stream));
    BK(cudaStreamSynchronize(b->stream));
    int64_t rb = 0;
    for (int c = 0; c < b->nchains; c++) {
        if (st[c].err) return fail(st[c].err, "chain " + std::to_string(c) + " reported status " + std::to_string(st[c].err));
        if (trials) trials[c] = st[c].trials;
        if (accepted) accepted[c] = st[c].accepted;
        if (etot) etot[c] = st[c].etot;
        rb += st[c].rebuilds;
    }
    b->rebuilds_seen = rb;
    return MCG_OK;
}

int mcg_batch_energy_fp64(mcg_batch* b, double* e) {
    if (!b || !e) return fail(MCG_EINVAL, "null argument");
    k_batch_energy64<<<b->ntiles, ETILE, 0, b->stream>>>(b->d_chains, b->d_tile_chain, b->d_tile_first, b->d_M, b->d_prm,
                                                         b->cut64, b->d_part);
    BK(cudaGetLastError());
    std::vector<double> part(b->ntiles);
    std::vector<int> tc(b->ntiles);
    BK(cudaMemcpyAsync(part.data(), b->d_part, sizeof(double) * b->ntiles, cudaMemcpyDeviceToHost, b->stream));
    BK(cudaMemcpyAsync(tc.data(), b->d_tile_chain, sizeof(int) * b->ntiles, cudaMemcpyDeviceToHost, b->stream));
    BK(cudaStreamSynchronize(b->stream));
    for (int c = 0; c < b->nchains; c++) e[c] = 0.0;
    for (int t = 0; t < b->ntiles; t++) e[tc[t]] += part[t];
    b->launches += 1;
    return MCG_OK;
}

int mcg_batch_get_coords(mcg_batch* b, int chain, double* x, double* y, double* z) {
    if (!b || chain < 0 || chain >= b->nchains || !x || !y || !z) return fail(MCG_EINVAL, "bad arguments");
    const ChainDev& C = b->chains[chain];
    int n = C.nres * C.apr;
    std::vector<ulonglong4_32a> M(n);
    BK(cudaMemcpyAsync(M.data(), b->d_M + C.atom0, sizeof(ulonglong4_32a) * n, cudaMemcpyDeviceToHost, b->stream));
    BK(cudaStreamSynchronize(b->stream));
    for (int i = 0; i < n; i++) { x[i] = host_view(M[i].x, C.L[0]); y[i] = host_view(M[i].y, C.L[1]); z[i] = host_view(M[i].z, C.L[2]); }
    return MCG_OK;
}

int mcg_batch_set_coords(mcg_batch* b, int chain, const double* x, const double* y, const double* z) {
    if (!b || chain < 0 || chain >= b->nchains || !x || !y || !z) return fail(MCG_EINVAL, "bad arguments");
    const ChainDev& C = b->chains[chain];
    int n = C.nres * C.apr;
    std::vector<ulonglong4_32a> M(n);
    std::vector<uint4> F(n);
    for (int i = 0; i < n; i++) {
        if (!std::isfinite(x[i]) || !std::isfinite(y[i]) || !std::isfinite(z[i])) return fail(MCG_EINVAL, "non-finite coordinate");
        M[i].x = host_master(x[i], C.rL[0]); M[i].y = host_master(y[i], C.rL[1]); M[i].z = host_master(z[i], C.rL[2]); M[i].w = 0;
        F[i] = make_uint4((uint32_t)(M[i].x >> 32), (uint32_t)(M[i].y >> 32), (uint32_t)(M[i].z >> 32), (uint32_t)(i % C.apr));
    }
    BK(cudaMemcpyAsync(b->d_M + C.atom0, M.data(), sizeof(ulonglong4_32a) * n, cudaMemcpyHostToDevice, b->stream));
    BK(cudaMemcpyAsync(b->d_F + C.atom0, F.data(), sizeof(uint4) * n, cudaMemcpyHostToDevice, b->stream));
    int r = b->launch_build();
    if (r) return r;
    std::vector<double> e(b->nchains);
    r = mcg_batch_energy_fp64(b, e.data());
    if (r) return r;
    std::vector<ChainState> st(b->nchains);
    BK(cudaMemcpyAsync(st.data(), b->d_state, sizeof(ChainState) * b->nchains, cudaMemcpyDeviceToHost, b->stream));
    BK(cudaStreamSynchronize(b->stream));
    st[chain].etot = e[chain];
    BK(cudaMemcpyAsync(b->d_state + chain, &st[chain], sizeof(ChainState), cudaMemcpyHostToDevice, b->stream));
    BK(cudaStreamSynchronize(b->stream));
    return MCG_OK;
}

int mcg_batch_get_lists(mcg_batch* b, int chain, int* counts, int* entries, int64_t cap, int64_t* total) {
    if (!b || chain < 0 || chain >= b->nchains || !counts || !total) return fail(MCG_EINVAL, "bad arguments");
    const ChainDev& C = b->chains[chain];
    std::vector<int> nl(C.nres);
    BK(cudaMemcpyAsync(nl.data(), b->d_NL + C.res0, sizeof(int) * C.nres, cudaMemcpyDeviceToHost, b->stream));
    BK(cudaStreamSynchronize(b->stream));
    int64_t tot = 0;
    for (int r = 0; r < C.nres; r++) { counts[r] = nl[r]; tot += nl[r]; }
    *total = tot;
    if (entries && cap >= tot) {
        std::vector<uint16_t> rows((size_t)C.nres * b->G.cap);
        BK(cudaMemcpyAsync(rows.data(), b->d_LST + (size_t)C.res0 * b->G.cap, sizeof(uint16_t) * rows.size(),
                           cudaMemcpyDeviceToHost, b->stream));
        BK(cudaStreamSynchronize(b->stream));
        int64_t o = 0;
        for (int r = 0; r < C.nres; r++)
            for (int k = 0; k < nl[r]; k++) entries[o++] = rows[(size_t)r * b->G.cap + k];
    }
    return MCG_OK;
}

// ---- exact checkpoint of a batch ----------------------------------------------------------
// A chain's future is a function of its masters M, its Philox counter and statistics (ChainState:
// running energy, counters, dmax and the acceptances since the last dmax adjustment, the largest
// displacement since the last list build), its lists and the launch shape.  The lists are a
// deterministic function of the mirror positions at their build (FB: cells sorted by residue
// index), so the file holds FB, not the lists: loading rebuilds every chain's lists from its FB
// and then restores M, the mirror and the states.  The launch shape matters too (the speculation
// width sets how a move's pair terms are split over warps, so the FP32 sums' order), so it is saved
// and re-applied.  Layout: magic, sizes, launch shape, ChainDev[nchains] and BatchGeom (checked
// against the loading batch: same chains, options and Philox keys), ChainState[nchains],
// M[natoms], FB[natoms], FNV-1a checksum of all the preceding bytes.
static const char kCkptMagic[8] = {'M', 'C', 'G', 'B', 'C', 'K', 'P', '1'};

struct CkptHeader {
    char magic[8];
    int32_t version, nchains;
    int64_t natoms, nres;
    int32_t threads, ctas_per_sm, spec_cap, clusters;
};

static uint64_t fnv1a(uint64_t h, const void* p, size_t n) {
    const unsigned char* c = (const unsigned char*)p;
    for (size_t k = 0; k < n; k++) { h ^= c[k]; h *= 1099511628211ull; }
    return h;
}

// the chains' constants without the speculation width (a launch-shape setting)
static std::vector<ChainDev> chains_for_compare(const std::vector<ChainDev>& v) {
    std::vector<ChainDev> w(v);
    for (ChainDev& c : w) c.kspec = 0;
    return w;
}

int mcg_batch_save(mcg_batch* b, const char* path) {
    if (!b || !path) return fail(MCG_EINVAL, "null argument");
    const int64_t na = b->natoms;
    std::vector<ChainState> st(b->nchains);
    std::vector<ulonglong4_32a> M(na);
    std::vector<uint4> FB(na);
    BK(cudaMemcpyAsync(st.data(), b->d_state, sizeof(ChainState) * b->nchains, cudaMemcpyDeviceToHost, b->stream));
    BK(cudaMemcpyAsync(M.data(), b->d_M, sizeof(ulonglong4_32a) * na, cudaMemcpyDeviceToHost, b->stream));
    BK(cudaMemcpyAsync(FB.data(), b->d_FB, sizeof(uint4) * na, cudaMemcpyDeviceToHost, b->stream));
    BK(cudaStreamSynchronize(b->stream));
    CkptHeader h;
    memset(&h, 0, sizeof h);
    memcpy(h.magic, kCkptMagic, 8);
    h.version = 1;
    h.nchains = b->nchains;
    h.natoms = na;
    h.nres = b->nres;
    h.threads = b->threads;
    h.ctas_per_sm = b->ctas_per_sm;
    h.spec_cap = b->spec_cap;
    h.clusters = b->clusters;
    std::string tmp = std::string(path) + ".part";
    FILE* f = fopen(tmp.c_str(), "wb");
    if (!f) return fail(MCG_EIO, std::string("cannot write ") + tmp);
    uint64_t sum = 1469598103934665603ull;
    bool ok = true;
    auto put = [&](const void* p, size_t n) {
        sum = fnv1a(sum, p, n);
        ok = ok && fwrite(p, 1, n, f) == n;
    };
    put(&h, sizeof h);
    put(b->chains.data(), sizeof(ChainDev) * b->nchains);
    put(&b->G, sizeof(BatchGeom));
    put(st.data(), sizeof(ChainState) * b->nchains);
    put(M.data(), sizeof(ulonglong4_32a) * na);
    put(FB.data(), sizeof(uint4) * na);
    ok = ok && fwrite(&sum, 1, sizeof sum, f) == sizeof sum;
    ok = (fclose(f) == 0) && ok;
    if (!ok || std::rename(tmp.c_str(), path) != 0) {
        std::remove(tmp.c_str());
        return fail(MCG_EIO, std::string("cannot write ") + path);
    }
    return MCG_OK;
}

int mcg_batch_load(mcg_batch* b, const char* path) {
    if (!b || !path) return fail(MCG_EINVAL, "null argument");
    FILE* f = fopen(path, "rb");
    if (!f) return fail(MCG_EIO, std::string("cannot read ") + path);
    std::vector<unsigned char> buf;
    {
        unsigned char chunk[1 << 16];
        size_t n;
        while ((n = fread(chunk, 1, sizeof chunk, f)) > 0) buf.insert(buf.end(), chunk, chunk + n);
        fclose(f);
    }
    const int64_t na = b->natoms;
    const size_t need = sizeof(CkptHeader) + sizeof(ChainDev) * b->nchains + sizeof(BatchGeom) +
                        sizeof(ChainState) * b->nchains + (sizeof(ulonglong4_32a) + sizeof(uint4)) * na + sizeof(uint64_t);
    CkptHeader h;
    if (buf.size() < sizeof h) return fail(MCG_EIO, "checkpoint file is truncated");
    memcpy(&h, buf.data(), sizeof h);
    if (memcmp(h.magic, kCkptMagic, 8) != 0 || h.version != 1) return fail(MCG_EIO, "not a batch checkpoint file");
    if (h.nchains != b->nchains || h.natoms != na || h.nres != b->nres)
        return fail(MCG_EINVAL, "checkpoint is of a batch with other chain or atom counts");
    if (buf.size() != need) return fail(MCG_EIO, "checkpoint file has the wrong size (truncated or damaged)");
    uint64_t sum;
    memcpy(&sum, buf.data() + need - sizeof sum, sizeof sum);
    if (fnv1a(1469598103934665603ull, buf.data(), need - sizeof sum) != sum) return fail(MCG_EIO, "checkpoint checksum mismatch");
    size_t o = sizeof h;
    std::vector<ChainDev> saved(b->nchains);
    memcpy(saved.data(), buf.data() + o, sizeof(ChainDev) * b->nchains);
    o += sizeof(ChainDev) * b->nchains;
    BatchGeom G;
    memcpy(&G, buf.data() + o, sizeof G);
    o += sizeof G;
    {
        std::vector<ChainDev> a = chains_for_compare(saved), c = chains_for_compare(b->chains);
        if (memcmp(a.data(), c.data(), sizeof(ChainDev) * b->nchains) != 0 || memcmp(&G, &b->G, sizeof G) != 0)
            return fail(MCG_EINVAL, "checkpoint is of other chains or options (boxes, temperatures, moves, seed)");
    }
    if (h.threads != b->threads || h.ctas_per_sm != b->ctas_per_sm || h.spec_cap != b->spec_cap || h.clusters != b->clusters) {
        int r = b->reconfigure(h.threads, h.ctas_per_sm, h.spec_cap, h.clusters);
        if (r) return r;
    }
    for (int c = 0; c < b->nchains; c++)
        if (b->chains[c].kspec != saved[c].kspec) return fail(MCG_EINVAL, "checkpoint launch shape could not be re-applied");
    const ChainState* st = (const ChainState*)(buf.data() + o);
    o += sizeof(ChainState) * b->nchains;
    const ulonglong4_32a* M = (const ulonglong4_32a*)(buf.data() + o);
    o += sizeof(ulonglong4_32a) * na;
    const uint4* FB = (const uint4*)(buf.data() + o);
    // lists from the build positions, then the masters, the mirror and the states
    BK(cudaMemcpyAsync(b->d_F, FB, sizeof(uint4) * na, cudaMemcpyHostToDevice, b->stream));
    int r = b->launch_build(b->stream, 1);
    if (r) return r;
    std::vector<ChainState> chk(b->nchains);
    BK(cudaMemcpyAsync(chk.data(), b->d_state, sizeof(ChainState) * b->nchains, cudaMemcpyDeviceToHost, b->stream));
    BK(cudaStreamSynchronize(b->stream));
    for (int c = 0; c < b->nchains; c++)
        if (chk[c].err) return fail(chk[c].err, "neighbour list capacity exceeded (chain " + std::to_string(c) + ")");
    std::vector<uint4> F(na);
    for (const ChainDev& C : b->chains)
        for (int i = 0; i < C.nres * C.apr; i++) {
            const ulonglong4_32a& m = M[C.atom0 + i];
            F[C.atom0 + i] = make_uint4((uint32_t)(m.x >> 32), (uint32_t)(m.y >> 32), (uint32_t)(m.z >> 32), (uint32_t)(i % C.apr));
        }
    BK(cudaMemcpyAsync(b->d_M, M, sizeof(ulonglong4_32a) * na, cudaMemcpyHostToDevice, b->stream));
    BK(cudaMemcpyAsync(b->d_F, F.data(), sizeof(uint4) * na, cudaMemcpyHostToDevice, b->stream));
    BK(cudaMemcpyAsync(b->d_FB, FB, sizeof(uint4) * na, cudaMemcpyHostToDevice, b->stream));
    BK(cudaMemcpyAsync(b->d_state, st, sizeof(ChainState) * b->nchains, cudaMemcpyHostToDevice, b->stream));
    BK(cudaStreamSynchronize(b->stream));
    return MCG_OK;
}

int mcg_batch_update_lists(mcg_batch* b) {
    if (!b) return fail(MCG_EINVAL, "null handle");
    int r = b->launch_build();
    if (r) return r;
    BK(cudaStreamSynchronize(b->stream));
    return mcg_batch_stats(b, nullptr, nullptr, nullptr);
}

int64_t mcg_batch_natoms(mcg_batch* b) { return b ? b->natoms : 0; }

int mcg_batch_chain_natoms(mcg_batch* b, int chain) {
    if (!b || chain < 0 || chain >= b->nchains) return fail(MCG_EINVAL, "bad chain");
    return b->chains[chain].nres * b->chains[chain].apr;
}

int mcg_batch_counters(mcg_batch* b, int64_t* list_rebuilds, int64_t* kernel_launches) {
    if (!b) return fail(MCG_EINVAL, "null handle");
    int r = mcg_batch_stats(b, nullptr, nullptr, nullptr);
    if (r) return r;
    if (list_rebuilds) *list_rebuilds = b->rebuilds_seen;
    if (kernel_launches) *kernel_launches = b->launches;
    return MCG_OK;
}

}  // extern "C"
