// Group-pair form of the pruned Verlet rows and its energy kernel (see groups.hpp).
#include <algorithm>
#include <climits>
#include <string>
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
#define MCG_GROUP_G(GS_)                                                                                          \
    if (v == 0) { if (G.iso) { MCG_GROUP_ONE(GS_, true, 2, true) } else { MCG_GROUP_ONE(GS_, false, 2, true) } }   \
    else { if (G.iso) { MCG_GROUP_ONE(GS_, true, 3, false) } else { MCG_GROUP_ONE(GS_, false, 3, false) } }
    if (gmax <= 3) { MCG_GROUP_G(3) } else { MCG_GROUP_G(4) }
#undef MCG_GROUP_G
#undef MCG_GROUP_ONE
    return blocks;
}

}  // namespace mcg
