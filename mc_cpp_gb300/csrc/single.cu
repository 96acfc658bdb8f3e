// Single-system engine: the device side of FField_CUDA.
//
// Data layout in HBM (one system, n atoms):
//   pq[n]        double4_32a (x, y, z, q)      FP64 master coordinates + charge (32 B, aligned loads)
//   es[n]        double2 (eps, sig)        sqrt(eps*418.4) and MDBAS half-sigma
//   es14[n]      double2 (eps14, sig14)
//   fx[n]        uint4 (fx, fy, fz, parameter class)  fixed-point mirror for the mixed kernels
//   cls_of[n], cls[ncls]  parameter class of each atom and the classes' (q hi, q lo, eps, sig)
//   esf[n]       float2 (eps, sig)
//   nbr[n*cap]   int   Verlet rows: partners j > i from the front, j < i from the back
//   nup[n], nlo[n]
//   cell_*       cell list of the last build
//   exclusion CSR (stored rows, and the full-mode effective rows), 1-4 pairs and per-atom 1-4 CSR
//   part[]       FP64 per-block partial sums (scratch), reduced in a fixed order by one block
//
// Kernels (all launched on the handle's stream):
//   k_cell_assign / k_cell_scan / k_cell_scatter / k_cell_sort / k_build_rows   Verlet build
//   k_energy_list<P>   switch energy over the half list (warp per row)        FField_MDBAS.cpp:336-424
//   k_energy_all<P>    full energy over all pairs (triangular tile grid)      FField_MDBAS.cpp:194-265
//   k_energy_14<P>     1-4 pairs                                               FField_MDBAS.cpp:267-318,426-488
//   k_bonded           bonds, Urey-Bradley, angles, dihedrals, impropers       FField_MDBAS.cpp:490-786
//   k_finalize         fixed-order reduction of the partials into ener[10]
//   k_delta_e<P>       energy change of a moved atom set, one launch
//   k_commit           write accepted coordinates
#include <algorithm>
#include <array>
#include <map>
#include <cmath>
#include <cstring>
#include <numeric>
#include <vector>

#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include "engine.hpp"
#include "pair_math.cuh"
#include "single.hpp"

namespace mcg {

#define CK(call)                                                                              \
    do {                                                                                      \
        cudaError_t e_ = (call);                                                              \
        if (e_ != cudaSuccess) return fail(MCG_ECUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

constexpr int NB_BLOCKS = 152 * 4;   // grid of the list-driven kernels: 4 CTAs per SM
constexpr int NB_THREADS = 256;
constexpr int MAX_MOVED = 1024;
constexpr int SORT_MAX = 2048;       // cells larger than this are sorted by one thread
constexpr int CLS_MAX = 1024;        // parameter classes the mixed pair kernel keeps in shared memory

enum { PREC_F64 = 0, PREC_MIX = 1 };

// ------------------------------------------------------------------------------------------
// Verlet list build with a cell grid (replaces the O(N^2) List_nonBonded::update_verlet_list,
// List_nonBonded.cpp:836-915; same acceptance rule: r^2 <= (rc + skin)^2 in the reference's FP64
// arithmetic, not both frozen, not in the stored exclusion row of the lower index).
// Cells at least half the list radius wide: a neighbour within the radius lies within two cells
// along each axis, so an atom scans up to 5 x 5 x 5 cells (a whole axis when it has fewer than 5).
struct Grid {
    int nc[3];
    double lo[3], inv[3];   // PBC none: bounding-box origin and 1 / extent
    float csf[3];           // cell widths, rounded down
    int periodic;
};

__global__ void k_cell_assign(const double4_32a* __restrict__ pq, int n, PbcDev pbc, Grid g, int* cell_of,
                              int* cell_count) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double4_32a p = pq[i];
    double c[3] = {p.x, p.y, p.z};
    int idx[3];
    for (int k = 0; k < 3; k++) {
        double u;
        if (g.periodic) { u = c[k] * pbc.rL[k]; u -= floor(u); }
        else u = (c[k] - g.lo[k]) * g.inv[k];
        int v = (int)(u * g.nc[k]);
        idx[k] = min(max(v, 0), g.nc[k] - 1);
    }
    int cell = (idx[2] * g.nc[1] + idx[1]) * g.nc[0] + idx[0];
    cell_of[i] = cell;
    atomicAdd(&cell_count[cell], 1);
}

// Exclusive scan of cell counts by one block (cells are few: one per (rc+skin)^3 of volume).
__global__ void k_cell_scan(const int* __restrict__ cell_count, int ncell, int* cell_start, int* cell_fill) {
    __shared__ int sh[1024];
    __shared__ int carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (int base = 0; base < ncell; base += 1024) {
        int i = base + threadIdx.x;
        int v = i < ncell ? cell_count[i] : 0;
        sh[threadIdx.x] = v;
        __syncthreads();
        for (int o = 1; o < 1024; o <<= 1) {
            int t = threadIdx.x >= o ? sh[threadIdx.x - o] : 0;
            __syncthreads();
            sh[threadIdx.x] += t;
            __syncthreads();
        }
        if (i < ncell) { cell_start[i] = carry + sh[threadIdx.x] - v; cell_fill[i] = 0; }
        __syncthreads();
        if (threadIdx.x == 1023) carry += sh[1023];
        __syncthreads();
    }
    if (threadIdx.x == 0) cell_start[ncell] = carry;
}

__global__ void k_cell_scatter(const int* __restrict__ cell_of, int n, const int* __restrict__ cell_start,
                               int* cell_fill, int* cell_atoms) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int c = cell_of[i];
    int slot = atomicAdd(&cell_fill[c], 1);
    cell_atoms[cell_start[c] + slot] = i;
}

// Sort each cell's atoms ascending so rows come out in a deterministic order.
__global__ void k_cell_sort(const int* __restrict__ cell_start, int ncell, int* cell_atoms) {
    __shared__ int sh[SORT_MAX];
    int c = blockIdx.x;
    if (c >= ncell) return;
    int b = cell_start[c], e = cell_start[c + 1], m = e - b;
    if (m <= 1) return;
    if (m > SORT_MAX) {
        if (threadIdx.x == 0)
            for (int i = b + 1; i < e; i++) {
                int v = cell_atoms[i], k = i - 1;
                while (k >= b && cell_atoms[k] > v) { cell_atoms[k + 1] = cell_atoms[k]; k--; }
                cell_atoms[k + 1] = v;
            }
        return;
    }
    int m2 = 1;
    while (m2 < m) m2 <<= 1;
    for (int i = threadIdx.x; i < m2; i += blockDim.x) sh[i] = i < m ? cell_atoms[b + i] : 0x7fffffff;
    __syncthreads();
    for (int k = 2; k <= m2; k <<= 1)
        for (int j = k >> 1; j > 0; j >>= 1) {
            for (int i = threadIdx.x; i < m2; i += blockDim.x) {
                int l = i ^ j;
                if (l > i) {
                    bool up = (i & k) == 0;
                    int a = sh[i], bb = sh[l];
                    if ((a > bb) == up) { sh[i] = bb; sh[l] = a; }
                }
            }
            __syncthreads();
        }
    for (int i = threadIdx.x; i < m; i += blockDim.x) cell_atoms[b + i] = sh[i];
}

struct ListParams {
    double cutnb2;
    int cap;
    int maxspan;
    // periodic boxes: FP32 prefilter on the fixed-point mirrors.  A pair whose FP32 r^2 lies below
    // lo2 is inside, above hi2 outside; only the band between takes the reference's FP64 test.
    float Ls[3], Ll[3];
    float lo2, hi2;
    float reach2;   // rows of cells farther than this (squared, with a margin) are not scanned
};

__device__ __forceinline__ bool stored_excluded(int lo, int hi, const int* __restrict__ xs,
                                                const int* __restrict__ xd, int maxspan) {
    if (hi - lo > maxspan) return false;
    int b = xs[lo], e = xs[lo + 1];
    for (int k = b; k < e; k++) if (xd[k] == hi) return true;
    return false;
}

// One warp per atom i; lanes walk the candidates of the stencil cells 32 at a time.  In periodic
// boxes each candidate is first placed by its FP32 distance from the exact fixed-point mirrors
// (error ~2e-7 of (rc + skin)^2); the reference's FP64 distance decides only the pairs within 1e-4
// of the list radius, so the rows are the reference's sets at a fraction of the FP64 work (GB300's
// FP64 rate is 1/64 of FP32).
__global__ void __launch_bounds__(256) k_build_rows(const double4_32a* __restrict__ pq, const uint4* __restrict__ fx,
                                                    const uint8_t* __restrict__ frozen,
                                                    int n, PbcDev pbc, Grid g, ListParams lp,
                                                    const int* __restrict__ cell_of, const int* __restrict__ cell_start,
                                                    const int* __restrict__ cell_atoms, const int* __restrict__ xs,
                                                    const int* __restrict__ xd, int* nbr, int* nup, int* nlo,
                                                    int* max_row) {
    const int lane = threadIdx.x & 31;
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nwarps = (gridDim.x * blockDim.x) >> 5;
    const bool periodic = pbc.type != 0;
    for (int i = warp; i < n; i += nwarps) {
        double4_32a pi = pq[i];
        const uint4 xi = periodic ? fx[i] : make_uint4(0, 0, 0, 0);
        bool fi = frozen[i] != 0;
        const int c = cell_of[i];
        const int ctr[3] = {c % g.nc[0], (c / g.nc[0]) % g.nc[1], c / (g.nc[0] * g.nc[1])};
        // per axis: the offsets scanned, and the atom's place inside its cell (in cell widths) for
        // the distance from the atom to a cell d away along that axis.  FP32 throughout (FP64 here,
        // warp-uniform but at GB300's FP64 rate, had cost more than the candidate tests): pos is
        // off by ~1e-6 cell widths, inside the margin of lp.reach2.
        int dlo[3], dhi[3];
        bool whole[3];
        float pos[3];
        const uint32_t fi3[3] = {xi.x, xi.y, xi.z};
        const double ci[3] = {pi.x, pi.y, pi.z};
        for (int k = 0; k < 3; k++) {
            float p;
            if (g.periodic) {   // the mirror holds the box fraction in units of 2^-32
                p = (float)fi3[k] * 2.3283064365386963e-10f * (float)g.nc[k] - (float)ctr[k];
                if (p < -0.5f * g.nc[k]) p += (float)g.nc[k];       // fraction just below 1, stored as 0
                else if (p > 0.5f * g.nc[k]) p -= (float)g.nc[k];
            } else {
                p = (float)((ci[k] - g.lo[k]) * g.inv[k]) * (float)g.nc[k] - (float)ctr[k];
            }
            pos[k] = fminf(fmaxf(p, 0.f), 1.f);
            whole[k] = g.periodic && g.nc[k] < 5;
            if (whole[k]) { dlo[k] = -ctr[k]; dhi[k] = g.nc[k] - 1 - ctr[k]; }
            else if (g.periodic) { dlo[k] = -2; dhi[k] = 2; }
            else { dlo[k] = max(-2, -ctr[k]); dhi[k] = min(2, g.nc[k] - 1 - ctr[k]); }
        }
        auto gap2 = [&](int k, int d) -> float {   // squared lower bound on |displacement| along axis k
            if (whole[k] || d == 0) return 0.f;
            const float w = (d > 0 ? (float)(d - 1) + (1.f - pos[k]) : (float)(-d - 1) + pos[k]) * g.csf[k];
            return w * w;
        };
        int up = 0, lo = 0;
        int* row = nbr + (size_t)i * lp.cap;
        // candidates b .. e-1 of cell_atoms, four batches of 32 in flight per warp (the index load
        // and the gather behind it are the latency); rows keep the candidates' order
        auto scan = [&](int b, int e) {
            constexpr int U = 4;
            for (int base = b; base < e; base += 32 * U) {
                int jj[U];
                uint4 xj[U];
#pragma unroll
                for (int u = 0; u < U; u++) {
                    const int t = base + 32 * u + lane;
                    jj[u] = t < e ? cell_atoms[t] : -1;
                }
                if (periodic) {
#pragma unroll
                    for (int u = 0; u < U; u++) xj[u] = jj[u] >= 0 ? fx[jj[u]] : make_uint4(0, 0, 0, 0);
                }
#pragma unroll
                for (int u = 0; u < U; u++) {
                    if (base + 32 * u >= e) break;   // warp-uniform
                    const int j = jj[u];
                    bool ok_up = false, ok_lo = false;
                    if (j >= 0 && j != i) {
                        bool in;
                        float r2f = 0.0f;
                        if (periodic) {
                            const float dx = fixed_delta(xi.x, xj[u].x, lp.Ls[0], lp.Ll[0]);
                            const float dy = fixed_delta(xi.y, xj[u].y, lp.Ls[1], lp.Ll[1]);
                            const float dz = fixed_delta(xi.z, xj[u].z, lp.Ls[2], lp.Ll[2]);
                            r2f = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
                        }
                        if (periodic && r2f < lp.lo2) in = true;
                        else if (periodic && r2f > lp.hi2) in = false;
                        else {
                            double4_32a pj = pq[j];
                            in = ref64_dist2(pi.x, pi.y, pi.z, pj.x, pj.y, pj.z, pbc) <= lp.cutnb2;
                        }
                        if (in && !(fi && frozen[j])) {
                            int a = min(i, j), bb = max(i, j);
                            if (!stored_excluded(a, bb, xs, xd, lp.maxspan)) {
                                ok_up = j > i;
                                ok_lo = j < i;
                            }
                        }
                    }
                    unsigned bu = __ballot_sync(0xffffffffu, ok_up);
                    unsigned bl = __ballot_sync(0xffffffffu, ok_lo);
                    unsigned lt = (1u << lane) - 1u;
                    if (ok_up) {
                        int p = up + __popc(bu & lt);
                        if (p + lo < lp.cap) row[p] = j;
                    }
                    if (ok_lo) {
                        int p = lo + __popc(bl & lt);
                        if (up + p < lp.cap) row[lp.cap - 1 - p] = j;
                    }
                    up += __popc(bu);
                    lo += __popc(bl);
                }
            }
        };
        // the stencil's rows of cells along x (at most 5 x 5), one per lane: rows and end cells out
        // of reach are dropped, and each row becomes one or two contiguous ranges of cell_atoms
        const int ny = dhi[1] - dlo[1] + 1, nrow = ny * (dhi[2] - dlo[2] + 1);
        int rb0 = 0, re0 = 0, rb1 = 0, re1 = 0;
        bool keep = false;
        if (lane < nrow) {
            const int dy = dlo[1] + lane % ny, dz = dlo[2] + lane / ny;
            const float left = lp.reach2 - gap2(2, dz) - gap2(1, dy);
            if (left >= 0.f) {
                keep = true;
                int x0 = dlo[0], x1 = dhi[0];
                while (x0 < 0 && gap2(0, x0) > left) x0++;
                while (x1 > 0 && gap2(0, x1) > left) x1--;
                int y = ctr[1] + dy, z = ctr[2] + dz;
                if (g.periodic) { y = (y + g.nc[1]) % g.nc[1]; z = (z + g.nc[2]) % g.nc[2]; }
                const int rowc = (z * g.nc[1] + y) * g.nc[0];
                int a0 = ctr[0] + x0, a1 = ctr[0] + x1;   // both wrap only on a whole axis, which has none
                if (a0 < 0) { rb1 = cell_start[rowc + a0 + g.nc[0]]; re1 = cell_start[rowc + g.nc[0]]; a0 = 0; }
                if (a1 >= g.nc[0]) { rb1 = cell_start[rowc]; re1 = cell_start[rowc + a1 - g.nc[0] + 1]; a1 = g.nc[0] - 1; }
                rb0 = cell_start[rowc + a0];
                re0 = cell_start[rowc + a1 + 1];
            }
        }
        // rows in lane order (z outer, y inner), the wrapped part of a row first
        for (unsigned km = __ballot_sync(0xffffffffu, keep); km; km &= km - 1) {
            const int r = __ffs(km) - 1;
            const int b1 = __shfl_sync(0xffffffffu, rb1, r), e1 = __shfl_sync(0xffffffffu, re1, r);
            const int b0 = __shfl_sync(0xffffffffu, rb0, r), e0 = __shfl_sync(0xffffffffu, re0, r);
            if (e1 > b1) scan(b1, e1);
            scan(b0, e0);
        }
        if (lane == 0) {
            nup[i] = up;
            nlo[i] = lo;
            atomicMax(max_row, up + lo);
        }
    }
}

// ------------------------------------------------------------------------------------------
// Energies.
struct AtomsDev {
    const double4_32a* pq;
    const double2* es;
    const double2* es14;
    const uint4* fx;
    const float2* esf;
    const float2* esf14;
    const float2* qf;     // charge as float-float (hi, lo)
    float Ls[3], Lsl[3];  // box / 2^32 as float-float (mixed displacement scale)
};

template <int P>
__device__ __forceinline__ void pair_energy(const AtomsDev& A, const PbcDev& pbc, const CutDev& cut, bool fourteen,
                                            double4_32a pi, uint4 fi, int i, double4_32a pj, uint4 fj, int j,
                                            bool apply_cut, double& el, double& vd) {
    if (P == PREC_F64) {
        double r2 = ref64_dist2(pi.x, pi.y, pi.z, pj.x, pj.y, pj.z, pbc);
        el = 0.0; vd = 0.0;
        if (apply_cut && r2 > cut.c2) return;
        double2 a = fourteen ? A.es14[i] : A.es[i];
        double2 b = fourteen ? A.es14[j] : A.es[j];
        ref64_pair(r2, pi.w, pj.w, a.x, b.x, a.y, b.y, apply_cut, cut, el, vd);
    } else {
        float dx, dy, dz;
        if (pbc.type != 0) {
            dx = fixed_delta(fi.x, fj.x, A.Ls[0], A.Lsl[0]);
            dy = fixed_delta(fi.y, fj.y, A.Ls[1], A.Lsl[1]);
            dz = fixed_delta(fi.z, fj.z, A.Ls[2], A.Lsl[2]);
        } else {
            dx = (float)(pj.x - pi.x); dy = (float)(pj.y - pi.y); dz = (float)(pj.z - pi.z);
        }
        float r2 = dx * dx + dy * dy + dz * dz;
        el = 0.0; vd = 0.0;
        if (apply_cut && r2 > cut.c2f) return;
        float2 a = fourteen ? A.esf14[i] : A.esf[i];
        float2 b = fourteen ? A.esf14[j] : A.esf[j];
        float s = a.y + b.y;
        float2 qa = A.qf[i], qb = A.qf[j];
        float qh, ql;
        ff_mul(qa.x, qa.y, qb.x, qb.y, qh, ql);
        float e1, v1;
        mixed_pair(r2, qh, ql, a.x * b.x, s * s, apply_cut, cut, e1, v1);
        el = e1; vd = v1;
    }
}

// Switch energy over the half list: a warp per row i, lanes over its j > i entries.
template <int P>
__global__ void __launch_bounds__(NB_THREADS) k_energy_list(AtomsDev A, int n, PbcDev pbc, CutDev cut,
                                                            const int* __restrict__ nbr, const int* __restrict__ nup,
                                                            int cap, double* part) {
    const int lane = threadIdx.x & 31;
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nwarps = (gridDim.x * blockDim.x) >> 5;
    double sel = 0.0, svd = 0.0;
    for (int i = warp; i < n; i += nwarps) {
        double4_32a pi = A.pq[i];
        uint4 fi = P == PREC_MIX ? A.fx[i] : make_uint4(0, 0, 0, 0);
        const int* row = nbr + (size_t)i * cap;
        int m = nup[i];
        F32Acc fe, fv;
        for (int k = lane; k < m; k += 32) {
            int j = row[k];
            double4_32a pj = P == PREC_F64 ? A.pq[j] : make_double4_32a(0, 0, 0, 0);
            uint4 fj = P == PREC_MIX ? A.fx[j] : make_uint4(0, 0, 0, 0);
            if (P == PREC_MIX && pbc.type == 0) pj = A.pq[j];
            double el, vd;
            pair_energy<P>(A, pbc, cut, false, pi, fi, i, pj, fj, j, true, el, vd);
            if (P == PREC_F64) { sel += el; svd += vd; }
            else { fe.add((float)el); fv.add((float)vd); }
        }
        if (P == PREC_MIX) { sel += fe.value(); svd += fv.value(); }
    }
    block_reduce2(sel, svd, part + 2 * blockIdx.x);
}

// One batch of U entries per lane of row i: the pair terms of k_energy_list_mix.
template <int U, bool ISO, bool TYPED>
__device__ __forceinline__ void mix_batch(const int (&j)[U], const uint4 (&fj)[U], float4 (&pj)[U], const float4* s_cls,
                                          int i, uint4 fi, float4 pi, int k0, int m, float Ls0, float Ls1, float Ls2,
                                          float Ll0, float Ll1, float Ll2, float L2h, float L2l, float c2, float n2,
                                          float k3, float& ch, float& cl, float& vs) {
    // the batch's terms are summed in FP32 (at most U per lane), then added to the row sums once;
    // a slot past the row's end or beyond rc takes r^2 = rc^2, where the switch polynomial is 0
    float th = 0.f, tl = 0.f;
#pragma unroll
    for (int u = 0; u < U; u++) {
        if (k0 + u * 32 >= m) break;   // warp-uniform: this and later slots are past the row
        if (TYPED) pj[u] = s_cls[fj[u].w];
        float r2;
        if (ISO) {
            const float ux = __int2float_rn((int)(fj[u].x - fi.x)), uy = __int2float_rn((int)(fj[u].y - fi.y)),
                        uz = __int2float_rn((int)(fj[u].z - fi.z));
            const float r2u = fmaf(ux, ux, fmaf(uy, uy, uz * uz));
            r2 = fmaf(r2u, L2h, r2u * L2l);
        } else {
            const float dx = fixed_delta(fi.x, fj[u].x, Ls0, Ll0), dy = fixed_delta(fi.y, fj[u].y, Ls1, Ll1),
                        dz = fixed_delta(fi.z, fj[u].z, Ls2, Ll2);
            r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
        }
        r2 = (j[u] != i && r2 <= c2) ? r2 : c2;
        float rinv = rsqrtf(r2);
        rinv = rinv * fmaf(-0.5f * r2 * rinv, rinv, 1.5f);   // one Newton step
        const float uu = fmaxf(r2, n2);
        const float a = c2 - uu;
        const float f = a * a * fmaf(2.0f, uu, k3);
        const float g = rinv * f;
        th = fmaf(pj[u].x, g, th);
        tl = fmaf(pj[u].y, g, tl);
        const float y = (pi.w + pj[u].w) * rinv;
        const float x2 = y * y;
        const float x6 = x2 * x2 * x2;
        vs = fmaf(pj[u].z, fmaf(x6, x6, -x6) * f, vs);
    }
    float sm, er;
    two_sum(ch, th, sm, er);
    ch = sm;
    cl += tl + er;
}

// Mixed-precision switched energy over the half list for periodic boxes: the pair kernel.  A warp
// per row i, lanes over its j > i entries.  One 16-byte load per list entry (the fixed-point
// position: exact minimum-image displacement by 32-bit wrap-around, scaled by a float-float box
// length) and one 16-byte load per pair inside the cutoff (charge as float-float, eps, sig).
// The row's sums are factored: each lane sums q_j g (g = S(r^2)/r, float-float by TwoSum) and
// eps_j l S (l = x^12 - x^6, FP32) over its entries of row i, and at the row's end multiplies them
// by q_i (float-float) and eps_i into float-float totals; no FP64 arithmetic until the block sum.
// The switch is formed unscaled as A^2 B with A = rc^2 - u, B = 2u + rc^2 - 3 ron^2 and u = r^2
// raised to ron^2; inv_f1 = 1 / (that FP32 polynomial at ron^2) scales the block sums, so inner
// pairs have S = 1 exactly.  Same terms as mixed_pair (unscaled, k_finalize scales).
// U list entries in flight per lane; MINB resident CTAs per SM requested from the register
// allocator (occupancy against registers); the engine times the variants once and keeps the fastest.
// Without the class table (TYPED below), both gathers of an entry (position and parameters) are
// issued together, unconditionally: over pruned rows ~88% of the entries lie within rc, so the
// parameter load is rarely wasted and the two dependent gather phases become one.  A padded slot (past the row's end) reads atom i itself
// and is masked by its index.  Slots wholly past the row's end are skipped by a warp-uniform test.
// ISO (cubic boxes): r^2 is summed in fixed-point units (exact integer differences converted to
// FP32) and scaled once by the float-float square of the unit length, two instructions per entry
// instead of a float-float scale per axis.
// TYPED: the atoms' parameters come from a table of the system's distinct (q, eps, sig) classes
// in shared memory, indexed by the class the fixed-point mirror carries in w, so an entry costs
// one global gather (its position) instead of two.
template <int U, int MINB, bool ISO, bool TYPED>
__global__ void __launch_bounds__(NB_THREADS, MINB) k_energy_list_mix(const uint4* __restrict__ fx, const float4* __restrict__ prm,
                                                                      const float4* __restrict__ cls, int ncls,
                                                                      int n, float Ls0, float Ls1, float Ls2, float Ll0,
                                                                      float Ll1, float Ll2, float L2h, float L2l,
                                                                      CutDev cut, double inv_f1,
                                                                      const int* __restrict__ nbr,
                                                                      const int* __restrict__ nup, int cap, double* part) {
    extern __shared__ float4 s_cls[];
    if (TYPED) {
        for (int c = threadIdx.x; c < ncls; c += blockDim.x) s_cls[c] = cls[c];
        __syncthreads();
    }
    const int lane = threadIdx.x & 31;
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nwarps = (gridDim.x * blockDim.x) >> 5;
    const float c2 = cut.c2f, n2 = cut.n2f, k3 = c2 - 3.0f * n2;
    float EH = 0.0f, EL = 0.0f, VH = 0.0f, VL = 0.0f;   // this lane's totals, float-float
    for (int i = warp; i < n; i += nwarps) {
        const uint4 fi = fx[i];
        const float4 pi = prm[i];        // (q hi, q lo, eps, sig)
        const int* row = nbr + (size_t)i * cap;
        const int m = nup[i];
        float ch = 0.0f, cl = 0.0f, vs = 0.0f;
        for (int k0 = 0; k0 < m; k0 += 32 * U) {
            int j[U];
            uint4 fj[U];
            float4 pj[U];
#pragma unroll
            for (int u = 0; u < U; u++) {
                const int k = k0 + u * 32 + lane;
                j[u] = k < m ? row[k] : i;
            }
#pragma unroll
            for (int u = 0; u < U; u++) {
                fj[u] = fx[j[u]];
                if (!TYPED) pj[u] = prm[j[u]];
            }
            mix_batch<U, ISO, TYPED>(j, fj, pj, s_cls, i, fi, pi, k0, m, Ls0, Ls1, Ls2, Ll0, Ll1, Ll2, L2h, L2l, c2, n2,
                                     k3, ch, cl, vs);
        }
        mix_row_flush(pi, ch, cl, vs, EH, EL, VH, VL);
    }
    block_reduce2(((double)EH + (double)EL) * inv_f1, ((double)VH + (double)VL) * inv_f1, part + 2 * blockIdx.x);
}

// Dynamic pruning of the half Verlet rows for the pair kernel: row i keeps, in its order, the
// partners j > i whose FP32 distance (the pair kernel's own fixed-point displacement) lies within
// the prune radius rp at the current positions.  While no atom has moved more than (rp - rc) / 2
// since, every list pair within rc is still in the pruned rows, so the pair kernel sums the same
// pairs over ~30% fewer entries (rc + skin = 14 A list, rp = 12.5 A).  The reference's stale-list
// set is kept: pruning only removes pairs, never adds one the Verlet build left out.  A warp per
// row, U entries in flight per lane, survivors compacted by ballot.
constexpr int PRUNE_U = 4;

__global__ void __launch_bounds__(NB_THREADS) k_prune_rows(const uint4* __restrict__ fx, int n, float Ls0, float Ls1,
                                                        float Ls2, float Ll0, float Ll1, float Ll2, float rp2,
                                                        const int* __restrict__ nbr, const int* __restrict__ nup,
                                                        int cap, int* __restrict__ prn, int* __restrict__ pnup,
                                                        unsigned long long* kept_total) {
    const int lane = threadIdx.x & 31;
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nwarps = (gridDim.x * blockDim.x) >> 5;
    const unsigned below = (1u << lane) - 1u;
    unsigned long long kept = 0;
    for (int i = warp; i < n; i += nwarps) {
        const uint4 fi = fx[i];
        const int* row = nbr + (size_t)i * cap;
        int* out = prn + (size_t)i * cap;
        const int m = nup[i];
        int w = 0;
        for (int k0 = 0; k0 < m; k0 += 32 * PRUNE_U) {
            int j[PRUNE_U];
            uint4 fj[PRUNE_U];
#pragma unroll
            for (int u = 0; u < PRUNE_U; u++) {
                const int k = k0 + u * 32 + lane;
                j[u] = k < m ? row[k] : -1;
            }
#pragma unroll
            for (int u = 0; u < PRUNE_U; u++) fj[u] = j[u] >= 0 ? fx[j[u]] : fi;
#pragma unroll
            for (int u = 0; u < PRUNE_U; u++) {
                const float dx = fixed_delta(fi.x, fj[u].x, Ls0, Ll0), dy = fixed_delta(fi.y, fj[u].y, Ls1, Ll1),
                            dz = fixed_delta(fi.z, fj[u].z, Ls2, Ll2);
                const bool keep = j[u] >= 0 && fmaf(dx, dx, fmaf(dy, dy, dz * dz)) <= rp2;
                const unsigned b = __ballot_sync(0xffffffffu, keep);
                if (keep) out[w + __popc(b & below)] = j[u];
                w += __popc(b);
            }
        }
        if (lane == 0) {
            pnup[i] = w;
            kept += (unsigned long long)w;
        }
    }
    if (lane == 0 && kept) atomicAdd(kept_total, kept);
}

// Full energy: all pairs j > i not in the full-mode exclusion row of i, no cutoff.  Triangular
// grid of TILE x TILE blocks; each thread owns one i and walks a shared-memory j tile with the
// reference's sorted-row cursor (FField_MDBAS.cpp:227-234).
constexpr int TILE = 128;

template <int P>
__global__ void __launch_bounds__(TILE) k_energy_all(AtomsDev A, int n, PbcDev pbc, CutDev cut,
                                                     const int* __restrict__ fxs, const int* __restrict__ fxd,
                                                     int ntile, double* part) {
    __shared__ double4_32a spq[TILE];
    __shared__ uint4 sfx[TILE];
    // block -> (I, J) with I <= J, row-major over the upper triangle
    int b = blockIdx.x;
    int I = 0;
    while (b >= ntile - I) { b -= ntile - I; I++; }
    int J = I + b;
    int i = I * TILE + threadIdx.x;
    int jt = J * TILE + threadIdx.x;
    if (jt < n) {
        spq[threadIdx.x] = A.pq[jt];
        if (P == PREC_MIX) sfx[threadIdx.x] = A.fx[jt];
    }
    __syncthreads();
    double sel = 0.0, svd = 0.0;
    if (i < n) {
        double4_32a pi = A.pq[i];
        uint4 fi = P == PREC_MIX ? A.fx[i] : make_uint4(0, 0, 0, 0);
        int xb = fxs[i], xe = fxs[i + 1];
        int cur = xb;
        int j0 = max(J * TILE, i + 1);
        while (cur < xe && fxd[cur] < j0) cur++;
        int jend = min(n, J * TILE + TILE);
        F32Acc fe, fv;
        for (int j = j0; j < jend; j++) {
            if (cur < xe && fxd[cur] == j) { cur++; continue; }
            int t = j - J * TILE;
            double el, vd;
            pair_energy<P>(A, pbc, cut, false, pi, fi, i, spq[t], P == PREC_MIX ? sfx[t] : make_uint4(0, 0, 0, 0), j,
                           false, el, vd);
            if (P == PREC_F64) { sel += el; svd += vd; }
            else { fe.add((float)el); fv.add((float)vd); }
        }
        if (P == PREC_MIX) { sel = fe.value(); svd = fv.value(); }
    }
    block_reduce2(sel, svd, part + 2 * blockIdx.x);
}

template <int P>
__global__ void k_energy_14(AtomsDev A, PbcDev pbc, CutDev cut, const int2* __restrict__ p14, int n14, double* part) {
    double sel = 0.0, svd = 0.0;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n14; k += gridDim.x * blockDim.x) {
        int2 p = p14[k];
        double el, vd;
        uint4 fi = P == PREC_MIX ? A.fx[p.x] : make_uint4(0, 0, 0, 0);
        uint4 fj = P == PREC_MIX ? A.fx[p.y] : make_uint4(0, 0, 0, 0);
        pair_energy<P>(A, pbc, cut, true, A.pq[p.x], fi, p.x, A.pq[p.y], fj, p.y, cut.mode == 1, el, vd);
        sel += el; svd += vd;
    }
    block_reduce2(sel, svd, part + 2 * blockIdx.x);
}

// ---- bonded terms (FP64, device math library) ---------------------------------------------
struct BondedDev {
    const BondT* bonds; int nb;
    const BondT* ubs; int nu;
    const AngleT* angles; int na;
    const TorsT* dihes; int nd;
    const TorsT* imprs; int ni;
};

__device__ __forceinline__ void crd(const double4_32a* pq, int i, double c[3]) {
    double4_32a p = pq[i]; c[0] = p.x; c[1] = p.y; c[2] = p.z;
}
__device__ __forceinline__ void apply_pbc(double d[3], const PbcDev& p) {
    if (p.type != 0) for (int k = 0; k < 3; k++) d[k] = ref64_mic(d[k], p.L[k], p.rL[k]);
}

// crd_of: coordinates of atom i, with moved atoms taken from the proposal.
struct CrdSrc {
    const double4_32a* pq;
    const int* mv_idx; const double* mv_xyz; int m;   // sorted moved atoms (may be m = 0)
    __device__ __forceinline__ void get(int i, double c[3]) const {
        int lo = 0, hi = m - 1;
        while (lo <= hi) {
            int mid = (lo + hi) >> 1, v = mv_idx[mid];
            if (v == i) { c[0] = mv_xyz[3 * mid]; c[1] = mv_xyz[3 * mid + 1]; c[2] = mv_xyz[3 * mid + 2]; return; }
            if (v < i) lo = mid + 1; else hi = mid - 1;
        }
        crd(pq, i, c);
    }
};

__device__ double bond_e(const BondT& b, const CrdSrc& S, const PbcDev& pbc, bool morse_ok) {
    double di[3], dj[3];
    S.get(b.a, di); S.get(b.b, dj);
    double d = sqrt(ref64_dist2(di[0], di[1], di[2], dj[0], dj[1], dj[2], pbc));
    if (morse_ok && b.type == 1) {
        double ma = exp(-b.beta * (d - b.r0));
        return b.k * (ma * ma - 2. * ma) + b.k;
    }
    return 0.5 * b.k * (d - b.r0) * (d - b.r0);
}

__device__ double angle_e(const AngleT& a, const CrdSrc& S, const PbcDev& pbc) {
    double di[3], dj[3], dk[3], dab[3], dbc[3];
    S.get(a.a, di); S.get(a.b, dj); S.get(a.c, dk);
    double rab = sqrt(ref64_dist2(di[0], di[1], di[2], dj[0], dj[1], dj[2], pbc, dab));
    double rbc = sqrt(ref64_dist2(dk[0], dk[1], dk[2], dj[0], dj[1], dj[2], pbc, dbc));
    double cost = (dab[0] * dbc[0] + dab[1] * dbc[1] + dab[2] * dbc[2]) / (rab * rbc);
    double th = acos(cost) - a.theta0;
    return 0.5 * a.k * th * th;
}

__device__ double tors_e(const TorsT& t, const CrdSrc& S, const PbcDev& pbc) {
    double di[3], dj[3], dk[3], dl[3], dab[3], dbc[3], dcd[3], pb[3], pc[3];
    S.get(t.a, di); S.get(t.b, dj); S.get(t.c, dk); S.get(t.d, dl);
    for (int k = 0; k < 3; k++) { dab[k] = di[k] - dj[k]; dcd[k] = dk[k] - dl[k]; }
    apply_pbc(dab, pbc); apply_pbc(dcd, pbc);
    double rbc = sqrt(ref64_dist2(dk[0], dk[1], dk[2], dj[0], dj[1], dj[2], pbc, dbc));
    pb[0] = dab[1] * dbc[2] - dab[2] * dbc[1];
    pb[1] = dab[2] * dbc[0] - dab[0] * dbc[2];
    pb[2] = dab[0] * dbc[1] - dab[1] * dbc[0];
    double rpb = sqrt(pb[0] * pb[0] + pb[1] * pb[1] + pb[2] * pb[2]);
    pc[0] = dbc[1] * dcd[2] - dbc[2] * dcd[1];
    pc[1] = dbc[2] * dcd[0] - dbc[0] * dcd[2];
    pc[2] = dbc[0] * dcd[1] - dbc[1] * dcd[0];
    double rpc = sqrt(pc[0] * pc[0] + pc[1] * pc[1] + pc[2] * pc[2]);
    double cosp = (pb[0] * pc[0] + pb[1] * pc[1] + pb[2] * pc[2]) / (rpb * rpc);
    double sinp = (dbc[0] * (pc[1] * pb[2] - pc[2] * pb[1]) + dbc[1] * (pb[0] * pc[2] - pb[2] * pc[0]) +
                   dbc[2] * (pc[0] * pb[1] - pc[1] * pb[0])) / (rpb * rpc * rbc);
    double phi = atan2(sinp, cosp);
    if (t.type == 2) {
        phi = phi - t.phi0;
        phi = phi - ref64_rint(phi / TWOPI) * TWOPI;
        return 0.5 * t.k * phi * phi;
    }
    return t.k * (1. + cos(t.mult * phi - t.phi0));
}

// part layout: 5 doubles per block (bond, ang, ub, dihe, impr)
__global__ void k_bonded(BondedDev B, PbcDev pbc, const double4_32a* __restrict__ pq, double* part) {
    double e[5] = {0, 0, 0, 0, 0};
    CrdSrc S{pq, nullptr, nullptr, 0};
    int total = B.nb + B.na + B.nu + B.nd + B.ni;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < total; k += gridDim.x * blockDim.x) {
        int t = k;
        if (t < B.nb) { e[0] += bond_e(B.bonds[t], S, pbc, true); continue; }
        t -= B.nb;
        if (t < B.na) { e[1] += angle_e(B.angles[t], S, pbc); continue; }
        t -= B.na;
        if (t < B.nu) { e[2] += bond_e(B.ubs[t], S, pbc, false); continue; }
        t -= B.nu;
        if (t < B.nd) { e[3] += tors_e(B.dihes[t], S, pbc); continue; }
        t -= B.nd;
        e[4] += tors_e(B.imprs[t], S, pbc);
    }
    __shared__ double sh[5][32];
    int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    for (int c = 0; c < 5; c++) {
        double v = warp_sum(e[c]);
        if (l == 0) sh[c][w] = v;
    }
    __syncthreads();
    if (threadIdx.x < 5) {
        double s = 0.0;
        for (int k = 0; k < (int)(blockDim.x >> 5); k++) s += sh[threadIdx.x][k];
        part[5 * blockIdx.x + threadIdx.x] = s;
    }
}

// Fixed-order reduction: one block.  nbp/n14p pairs of (el, vd) partials, bdp blocks of 5.
__global__ void k_finalize(const double* __restrict__ nb, int nnb, const double* __restrict__ p14, int n14,
                           const double* __restrict__ bd, int nbd, double* out) {
    __shared__ double sh[9][256];
    double acc[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    for (int k = threadIdx.x; k < nnb; k += blockDim.x) { acc[0] += nb[2 * k]; acc[1] += nb[2 * k + 1]; }
    for (int k = threadIdx.x; k < n14; k += blockDim.x) { acc[2] += p14[2 * k]; acc[3] += p14[2 * k + 1]; }
    for (int k = threadIdx.x; k < nbd; k += blockDim.x)
        for (int c = 0; c < 5; c++) acc[4 + c] += bd[5 * k + c];
    for (int c = 0; c < 9; c++) sh[c][threadIdx.x] = acc[c];
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) for (int c = 0; c < 9; c++) sh[c][threadIdx.x] += sh[c][threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        const double K = CHGCHARMM * KCALTOIU;
        double elec = K * sh[0][0];
        double vdw = 4.0 * sh[1][0];
        elec += K * sh[2][0];
        vdw += 4.0 * sh[3][0];
        double bond = sh[4][0], ang = sh[5][0], ub = sh[6][0], dihe = sh[7][0], impr = sh[8][0];
        double pot = elec + vdw + bond + ang + ub + dihe + impr;
        out[0] = pot + 0.0; out[1] = pot; out[2] = 0.0; out[3] = elec; out[4] = vdw;
        out[5] = bond; out[6] = ang; out[7] = ub; out[8] = dihe; out[9] = impr;
    }
}

// ------------------------------------------------------------------------------------------
// Energy change of a moved set.  Blocks b < m*S take moved atom mv[b / S] against slice b % S of
// its partners (Verlet row in switch mode, every atom in full mode) and of its 1-4 partners; block
// m*S evaluates the listed bonded terms.  Pairs with both atoms moved are counted once, by the
// lower index.  Spreading a row over S blocks matters most in FP64, which GB300 runs at about two
// lane operations per clock per SM: one block per moved atom left a water move's ~1,150 partners
// on three SMs.  The last block to finish sums the partials (a fixed tree over the block index,
// so de is reproducible) and writes de (iu).
struct MoveDev {
    int m;
    const int* idx;        // sorted moved atoms
    const double* xyz;     // their proposed coordinates (3 per atom)
    const int* terms;      // bonded terms touching them: (kind, index) pairs
    int nterms;
};

// A small proposal travels inside the launch (kernel parameter space, read through the constant
// cache), so that a trial move costs one launch and no copy; m = 0 means it was staged in device
// memory and MoveDev points there.
constexpr int INL_M = 32, INL_T = 96;
struct MoveInline {
    int m, nterms;
    int idx[INL_M];
    int terms[2 * INL_T];
    double xyz[3 * INL_M];
};

template <int P>
__global__ void __launch_bounds__(256) k_delta_e(AtomsDev A, int n, PbcDev pbc, CutDev cut, MoveDev mv,
                                                 const int* __restrict__ nbr, const int* __restrict__ nup,
                                                 const int* __restrict__ nlo, int cap,
                                                 const int* __restrict__ fxs, const int* __restrict__ fxd,
                                                 const int* __restrict__ c14s, const int* __restrict__ c14d,
                                                 BondedDev B, int S, double* part, unsigned* ticket, double* out,
                                                 const __grid_constant__ MoveInline inl) {
    __shared__ int s_idx[MAX_MOVED];
    __shared__ double s_xyz[3 * MAX_MOVED];
    __shared__ uint4 s_fx[MAX_MOVED];
    __shared__ bool s_last;
    if (inl.m > 0) { mv.m = inl.m; mv.idx = inl.idx; mv.xyz = inl.xyz; mv.terms = inl.terms; mv.nterms = inl.nterms; }
    const int m = mv.m;
    for (int k = threadIdx.x; k < m; k += blockDim.x) {
        s_idx[k] = mv.idx[k];
        double x = mv.xyz[3 * k], y = mv.xyz[3 * k + 1], z = mv.xyz[3 * k + 2];
        s_xyz[3 * k] = x; s_xyz[3 * k + 1] = y; s_xyz[3 * k + 2] = z;
        if (P == PREC_MIX) {
            uint4 f = A.fx[mv.idx[k]];
            if (pbc.type != 0) { f.x = to_fixed(x, pbc.rL[0]); f.y = to_fixed(y, pbc.rL[1]); f.z = to_fixed(z, pbc.rL[2]); }
            s_fx[k] = f;
        }
    }
    __syncthreads();
    auto slot = [&](int j) -> int {
        int lo = 0, hi = m - 1;
        while (lo <= hi) {
            int mid = (lo + hi) >> 1, v = s_idx[mid];
            if (v == j) return mid;
            if (v < j) lo = mid + 1; else hi = mid - 1;
        }
        return -1;
    };
    double del = 0.0, dvd = 0.0, dbd = 0.0;
    const bool sw = cut.mode == 1;
    if ((int)blockIdx.x < m * S) {
        const int ka = blockIdx.x / S;
        const int k0 = (blockIdx.x % S) * blockDim.x + threadIdx.x, kstep = S * blockDim.x;
        const int a = s_idx[ka];
        const double4_32a ao = A.pq[a];
        const double4_32a an = make_double4_32a(s_xyz[3 * ka], s_xyz[3 * ka + 1], s_xyz[3 * ka + 2], ao.w);
        const uint4 fo = P == PREC_MIX ? A.fx[a] : make_uint4(0, 0, 0, 0);
        const uint4 fn = P == PREC_MIX ? s_fx[ka] : make_uint4(0, 0, 0, 0);
        CutDev cutx = cut;   // full mode: no cutoff and no switch
        if (!sw) { cutx.c2f = 1.0e30f; cutx.n2f = 1.0e30f; }   // "no cutoff": finite, so c2 - 3 n2 stays finite
        float ma[3] = {0.f, 0.f, 0.f};   // the exact move of a, as the fixed-point mirror sees it
        if (P == PREC_MIX) {
            if (pbc.type != 0) {
                ma[0] = fixed_delta(fo.x, fn.x, A.Ls[0], A.Lsl[0]);
                ma[1] = fixed_delta(fo.y, fn.y, A.Ls[1], A.Lsl[1]);
                ma[2] = fixed_delta(fo.z, fn.z, A.Ls[2], A.Lsl[2]);
            } else {
                ma[0] = (float)(an.x - ao.x); ma[1] = (float)(an.y - ao.y); ma[2] = (float)(an.z - ao.z);
            }
        }
        auto visit = [&](int j, bool fourteen, bool apply_cut) {
            int sj = slot(j);
            if (sj >= 0 && j < a) return;       // counted by the lower index's block
            double4_32a jo = A.pq[j];
            uint4 gjo = P == PREC_MIX ? A.fx[j] : make_uint4(0, 0, 0, 0);
            double4_32a jn = jo;
            uint4 gjn = gjo;
            if (sj >= 0) { jn.x = s_xyz[3 * sj]; jn.y = s_xyz[3 * sj + 1]; jn.z = s_xyz[3 * sj + 2]; if (P == PREC_MIX) gjn = s_fx[sj]; }
            if (P == PREC_F64) {
                double e0, v0, e1, v1;
                pair_energy<P>(A, pbc, cut, fourteen, ao, fo, a, jo, gjo, j, apply_cut, e0, v0);
                pair_energy<P>(A, pbc, cut, fourteen, an, fn, a, jn, gjn, j, apply_cut, e1, v1);
                del += e1 - e0;
                dvd += v1 - v0;
            } else {
                // d_old = j_old - a_old, d_new = j_new - a_new = d_old - m
                float d[3], m[3];
                if (pbc.type != 0) {
                    d[0] = fixed_delta(fo.x, gjo.x, A.Ls[0], A.Lsl[0]); d[1] = fixed_delta(fo.y, gjo.y, A.Ls[1], A.Lsl[1]); d[2] = fixed_delta(fo.z, gjo.z, A.Ls[2], A.Lsl[2]);
                } else {
                    d[0] = (float)(jo.x - ao.x); d[1] = (float)(jo.y - ao.y); d[2] = (float)(jo.z - ao.z);
                }
                // d_new by minimum image; m = d_old - d_new is taken from the exact move of a when
                // only a moved (so the analytic difference keeps its accuracy), and the pair is
                // differenced directly when the move carries it across half the box
                float dn[3];
                if (pbc.type != 0) {
                    dn[0] = fixed_delta(fn.x, gjn.x, A.Ls[0], A.Lsl[0]); dn[1] = fixed_delta(fn.y, gjn.y, A.Ls[1], A.Lsl[1]); dn[2] = fixed_delta(fn.z, gjn.z, A.Ls[2], A.Lsl[2]);
                } else {
                    dn[0] = (float)(jn.x - an.x); dn[1] = (float)(jn.y - an.y); dn[2] = (float)(jn.z - an.z);
                }
                bool flip = false;
                if (sj >= 0) { m[0] = d[0] - dn[0]; m[1] = d[1] - dn[1]; m[2] = d[2] - dn[2]; }
                else {
                    m[0] = ma[0]; m[1] = ma[1]; m[2] = ma[2];
                    for (int t = 0; t < 3; t++) flip |= fabsf(d[t] - m[t] - dn[t]) > 1.0f;
                }
                float2 pa = fourteen ? A.esf14[a] : A.esf[a];
                float2 pb = fourteen ? A.esf14[j] : A.esf[j];
                float s = pa.y + pb.y;
                float2 qa = A.qf[a], qb = A.qf[j];
                float qh, ql;
                ff_mul(qa.x, qa.y, qb.x, qb.y, qh, ql);
                float qk = (float)(CHGCHARMM * KCALTOIU) * (qh + ql);
                int np_ = 0;
                if (!flip) {
                    dbd += (double)mixed_pair_delta(d[0], d[1], d[2], m[0], m[1], m[2], qk, 4.0f * pa.x * pb.x, s * s,
                                                    apply_cut ? cut : cutx, np_);
                } else {
                    float e0, v0, e1, v1;
                    const CutDev& cc = apply_cut ? cut : cutx;
                    const float u0 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2], u1 = dn[0] * dn[0] + dn[1] * dn[1] + dn[2] * dn[2];
                    e0 = v0 = e1 = v1 = 0.f;
                    if (!apply_cut || u0 <= cc.c2f) mixed_pair(u0, qh, ql, pa.x * pb.x, s * s, apply_cut, cc, e0, v0);
                    if (!apply_cut || u1 <= cc.c2f) mixed_pair(u1, qh, ql, pa.x * pb.x, s * s, apply_cut, cc, e1, v1);
                    dbd += (double)(CHGCHARMM * KCALTOIU) * ((double)e1 - (double)e0) + 4.0 * ((double)v1 - (double)v0);
                }
            }
        };
        if (sw) {
            const int* row = nbr + (size_t)a * cap;
            int u = nup[a], l = nlo[a];
            for (int k = k0; k < u + l; k += kstep) {
                int j = k < u ? row[k] : row[cap - 1 - (k - u)];
                visit(j, false, true);
            }
        } else {
            for (int j = k0; j < n; j += kstep) {
                if (j == a) continue;
                int lo_ = min(a, j), hi_ = max(a, j);
                bool ex = false;
                for (int k = fxs[lo_]; k < fxs[lo_ + 1]; k++) if (fxd[k] == hi_) { ex = true; break; }
                if (!ex) visit(j, false, false);
            }
        }
        for (int k = c14s[a] + k0; k < c14s[a + 1]; k += kstep) visit(c14d[k], true, sw);
    } else {
        CrdSrc S_old{A.pq, nullptr, nullptr, 0};
        CrdSrc S_new{A.pq, s_idx, s_xyz, m};
        for (int k = threadIdx.x; k < mv.nterms; k += blockDim.x) {
            int kind = mv.terms[2 * k], t = mv.terms[2 * k + 1];
            double e0 = 0, e1 = 0;
            if (kind == 0) { e0 = bond_e(B.bonds[t], S_old, pbc, true); e1 = bond_e(B.bonds[t], S_new, pbc, true); }
            else if (kind == 1) { e0 = angle_e(B.angles[t], S_old, pbc); e1 = angle_e(B.angles[t], S_new, pbc); }
            else if (kind == 2) { e0 = bond_e(B.ubs[t], S_old, pbc, false); e1 = bond_e(B.ubs[t], S_new, pbc, false); }
            else if (kind == 3) { e0 = tors_e(B.dihes[t], S_old, pbc); e1 = tors_e(B.dihes[t], S_new, pbc); }
            else { e0 = tors_e(B.imprs[t], S_old, pbc); e1 = tors_e(B.imprs[t], S_new, pbc); }
            dbd += e1 - e0;
        }
    }
    __shared__ double red[3];
    block_reduce2(del, dvd, red);
    {
        double v = warp_sum(dbd);
        __shared__ double sb[32];
        if ((threadIdx.x & 31) == 0) sb[threadIdx.x >> 5] = v;
        __syncthreads();
        if (threadIdx.x == 0) {
            double s = 0.0;
            for (int k = 0; k < (int)(blockDim.x >> 5); k++) s += sb[k];
            red[2] = s;
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        part[3 * blockIdx.x] = red[0];
        part[3 * blockIdx.x + 1] = red[1];
        part[3 * blockIdx.x + 2] = red[2];
        __threadfence();
        unsigned t = atomicAdd(ticket, 1u);
        s_last = (t == gridDim.x - 1);
    }
    __syncthreads();
    if (s_last) {   // uniform over the block
        __threadfence();
        double se = 0.0, sv = 0.0, sb = 0.0;
        for (unsigned b = threadIdx.x; b < gridDim.x; b += blockDim.x) {
            se += __ldcg(part + 3 * b);
            sv += __ldcg(part + 3 * b + 1);
            sb += __ldcg(part + 3 * b + 2);
        }
        block_reduce2(se, sv, red);
        __shared__ double rb[2];
        block_reduce2(sb, 0.0, rb);
        if (threadIdx.x == 0) {
            out[0] = CHGCHARMM * KCALTOIU * red[0] + 4.0 * red[1] + rb[0];
            out[1] = red[0]; out[2] = red[1]; out[3] = rb[0];
            *ticket = 0u;
        }
    }
}

template <int P>
__global__ void k_commit(int m, const int* idx, const double* xyz, double4_32a* pq, uint4* fx, PbcDev pbc,
                         const __grid_constant__ MoveInline inl) {
    if (inl.m > 0) { idx = inl.idx; xyz = inl.xyz; }
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= m) return;
    int a = idx[k];
    double4_32a p = pq[a];
    p.x = xyz[3 * k]; p.y = xyz[3 * k + 1]; p.z = xyz[3 * k + 2];
    pq[a] = p;
    if (pbc.type != 0) {
        uint4 f = fx[a];
        f.x = to_fixed(p.x, pbc.rL[0]); f.y = to_fixed(p.y, pbc.rL[1]); f.z = to_fixed(p.z, pbc.rL[2]);
        fx[a] = f;
    }
}

// Fixed-point mirror of every atom from the FP64 masters; w carries the atom's parameter class.
__global__ void k_fix_all(int n, const double4_32a* __restrict__ pq, const int* __restrict__ cls_of, uint4* fx, PbcDev pbc) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double4_32a p = pq[i];
    uint4 f;
    if (pbc.type != 0) { f.x = to_fixed(p.x, pbc.rL[0]); f.y = to_fixed(p.y, pbc.rL[1]); f.z = to_fixed(p.z, pbc.rL[2]); }
    else { f.x = f.y = f.z = 0; }
    f.w = (unsigned)cls_of[i];
    fx[i] = f;
}

// ==========================================================================================
// Host side of the engine.
template <typename T>
static int dalloc(T** p, size_t count) {
    *p = nullptr;
    if (count == 0) count = 1;
    cudaError_t e = cudaMalloc((void**)p, count * sizeof(T));
    if (e != cudaSuccess) return fail(MCG_ECUDA, std::string("cudaMalloc: ") + cudaGetErrorString(e));
    return MCG_OK;
}

template <typename T>
static int dupload(T** p, const std::vector<T>& v, cudaStream_t st) {
    int rc = dalloc(p, v.size());
    if (rc) return rc;
    if (!v.empty()) CK(cudaMemcpyAsync(*p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, st));
    return MCG_OK;
}

SingleEngine::~SingleEngine() { release(); }

void SingleEngine::release() {
    void* ptrs[] = {d_pq, d_es, d_es14, d_fx, d_esf, d_esf14, d_qf, d_prmf, d_frozen, d_xs, d_xd, d_fxs, d_fxd, d_p14, d_c14s,
                    d_c14d, d_bonds, d_ubs, d_angles, d_dihes, d_imprs, d_nbr, d_nup, d_nlo, d_cell_of,
                    d_cell_count, d_cell_start, d_cell_fill, d_cell_atoms, d_part, d_ticket, d_maxrow,
                    d_stage, d_prn, d_pnup, d_pkept, d_cls_of, d_cls};
    for (void* p : ptrs) if (p) cudaFree(p);
    for (cudaEvent_t& e : ev_prune) if (e) { cudaEventDestroy(e); e = nullptr; }
    if (h_stage) cudaFreeHost(h_stage);
    if (h_map) cudaFreeHost(h_map);
    h_map = nullptr; d_map = nullptr;
    if (stream) cudaStreamDestroy(stream);
    d_pq = nullptr; stream = nullptr; h_stage = nullptr;
}

int SingleEngine::init(const HostSystem& h) {
    hs = h;
    n = hs.n;
    CK(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
    pbc.type = hs.pbc;
    for (int k = 0; k < 3; k++) { pbc.L[k] = hs.L[k]; pbc.rL[k] = hs.rL[k]; }
    cut.mode = hs.cut;
    cut.c2 = hs.rc * hs.rc;
    cut.n2 = hs.ron * hs.ron;
    {
        double d = cut.c2 - cut.n2;
        cut.sw2 = 1. / (d * d * d);
    }
    cut.c2f = (float)cut.c2; cut.n2f = (float)cut.n2; cut.sw2f = (float)cut.sw2;
    std::vector<double4_32a> pq(n);
    std::vector<double2> es(n), es14(n);
    std::vector<float2> esf(n), esf14(n), qf(n);
    std::vector<float4> prmf(n);
    for (int i = 0; i < n; i++) {
        pq[i] = make_double4_32a(hs.x[i], hs.y[i], hs.z[i], hs.q[i]);
        es[i] = make_double2(hs.eps[i], hs.sig[i]);
        es14[i] = make_double2(hs.eps14[i], hs.sig14[i]);
        esf[i] = make_float2((float)hs.eps[i], (float)hs.sig[i]);
        esf14[i] = make_float2((float)hs.eps14[i], (float)hs.sig14[i]);
        float qh = (float)hs.q[i];
        qf[i] = make_float2(qh, (float)(hs.q[i] - (double)qh));
        prmf[i] = make_float4(qf[i].x, qf[i].y, esf[i].x, esf[i].y);
    }
    // parameter classes: the distinct (q hi, q lo, eps, sig) of the mixed pair kernel, in first-seen
    // order; more than CLS_MAX classes leave the table empty (the kernel gathers per atom)
    std::vector<int> cls_of(n, 0);
    std::vector<float4> cls;
    {
        std::map<std::array<uint32_t, 4>, int> seen;
        for (int i = 0; i < n && (int)cls.size() <= CLS_MAX; i++) {
            std::array<uint32_t, 4> key;
            memcpy(key.data(), &prmf[i], sizeof(float4));
            auto it = seen.find(key);
            if (it == seen.end()) {
                it = seen.emplace(key, (int)cls.size()).first;
                cls.push_back(prmf[i]);
            }
            cls_of[i] = it->second;
        }
        if ((int)cls.size() > CLS_MAX) {
            cls.clear();
            std::fill(cls_of.begin(), cls_of.end(), 0);
        }
        ncls = (int)cls.size();
    }
    int rc;
    if ((rc = dupload(&d_cls_of, cls_of, stream)) || (rc = dupload(&d_cls, cls, stream))) return rc;
    if ((rc = dupload(&d_pq, pq, stream)) || (rc = dupload(&d_es, es, stream)) || (rc = dupload(&d_es14, es14, stream)) ||
        (rc = dupload(&d_esf, esf, stream)) || (rc = dupload(&d_esf14, esf14, stream)) || (rc = dupload(&d_qf, qf, stream)) ||
        (rc = dupload(&d_prmf, prmf, stream)) ||
        (rc = dupload(&d_frozen, hs.frozen, stream)) || (rc = dupload(&d_xs, hs.exclStart, stream)) ||
        (rc = dupload(&d_xd, hs.exclData, stream)) || (rc = dupload(&d_fxs, hs.fexclStart, stream)) ||
        (rc = dupload(&d_fxd, hs.fexclData, stream)))
        return rc;
    if ((rc = dalloc(&d_fx, n))) return rc;
    if (uses_pair_variants() && ncls > 0) {   // groups of the group-pair kernels (residue runs of <= 4 atoms)
        if ((rc = grp.setup(hs.resid))) return rc;
        grp_setup = true;
    }
    // 1-4 pairs and their per-atom CSR (both directions) for the ΔE kernel
    n14 = (int)hs.pairs14.size() / 2;
    std::vector<int2> p14(n14);
    std::vector<std::vector<int>> adj(n);
    for (int k = 0; k < n14; k++) {
        p14[k] = make_int2(hs.pairs14[2 * k], hs.pairs14[2 * k + 1]);
        adj[p14[k].x].push_back(p14[k].y);
        adj[p14[k].y].push_back(p14[k].x);
    }
    std::vector<int> c14s(n + 1, 0), c14d;
    for (int i = 0; i < n; i++) { c14s[i] = (int)c14d.size(); c14d.insert(c14d.end(), adj[i].begin(), adj[i].end()); }
    c14s[n] = (int)c14d.size();
    if ((rc = dupload(&d_p14, p14, stream)) || (rc = dupload(&d_c14s, c14s, stream)) || (rc = dupload(&d_c14d, c14d, stream)))
        return rc;
    if ((rc = dupload(&d_bonds, hs.bonds, stream)) || (rc = dupload(&d_ubs, hs.ubs, stream)) ||
        (rc = dupload(&d_angles, hs.angles, stream)) || (rc = dupload(&d_dihes, hs.dihes, stream)) ||
        (rc = dupload(&d_imprs, hs.imprs, stream)))
        return rc;
    // per-atom bonded-term index for ΔE (kind, index)
    term_start.assign(n + 1, 0);
    std::vector<std::vector<int>> tl(n);
    auto addt = [&](int atom, int kind, int idx) { tl[atom].push_back(kind); tl[atom].push_back(idx); };
    for (int k = 0; k < (int)hs.bonds.size(); k++) { addt(hs.bonds[k].a, 0, k); addt(hs.bonds[k].b, 0, k); }
    for (int k = 0; k < (int)hs.angles.size(); k++) { const AngleT& a = hs.angles[k]; addt(a.a, 1, k); addt(a.b, 1, k); addt(a.c, 1, k); }
    for (int k = 0; k < (int)hs.ubs.size(); k++) { addt(hs.ubs[k].a, 2, k); addt(hs.ubs[k].b, 2, k); }
    for (int k = 0; k < (int)hs.dihes.size(); k++) { const TorsT& t = hs.dihes[k]; addt(t.a, 3, k); addt(t.b, 3, k); addt(t.c, 3, k); addt(t.d, 3, k); }
    for (int k = 0; k < (int)hs.imprs.size(); k++) { const TorsT& t = hs.imprs[k]; addt(t.a, 4, k); addt(t.b, 4, k); addt(t.c, 4, k); addt(t.d, 4, k); }
    term_data.clear();
    for (int i = 0; i < n; i++) { term_start[i] = (int)term_data.size() / 2; term_data.insert(term_data.end(), tl[i].begin(), tl[i].end()); }
    term_start[n] = (int)term_data.size() / 2;
    // scratch: partial sums and the ΔE ticket
    ntile = (n + TILE - 1) / TILE;
    size_t nparts = std::max<size_t>({(size_t)152 * 8, (size_t)ntile * (ntile + 1) / 2, (size_t)MAX_MOVED + 1});
    part_cap = nparts * 3 + 2 * 64 + 5 * 64 + 16;
    if ((rc = dalloc(&d_part, part_cap)) || (rc = dalloc(&d_ticket, 1)) ||
        (rc = dalloc(&d_maxrow, 1)))
        return rc;
    CK(cudaMemsetAsync(d_ticket, 0, sizeof(unsigned), stream));
    // staging for moves: idx (sorted), xyz, terms
    stage_bytes = (size_t)MAX_MOVED * (4 + 24) + 64 * 1024 * 8;
    CK(cudaMallocHost(&h_stage, stage_bytes));
    // results the host reads after a sync: de at [0, 4), the ten energy terms at [8, 18)
    CK(cudaHostAlloc((void**)&h_map, 32 * sizeof(double), cudaHostAllocMapped));
    CK(cudaHostGetDevicePointer((void**)&d_map, h_map, 0));
    if ((rc = dalloc((char**)&d_stage, stage_bytes))) return rc;
    k_fix_all<<<(n + 255) / 256, 256, 0, stream>>>(n, d_pq, d_cls_of, d_fx, pbc);
    CK(cudaGetLastError());
    host_x = hs.x; host_y = hs.y; host_z = hs.z;
    if (hs.cut == MCG_CUT_SWITCH) {
        if ((rc = build_list())) return rc;
    }
    CK(cudaStreamSynchronize(stream));
    return MCG_OK;
}

// The switched nonbonded kernel over the half list (FP64, or mixed: the dedicated pair kernel for
// periodic boxes).
int SingleEngine::launch_nonbonded(double* nbp) {
    AtomsDev A = atoms();
    if (hs.prec == MCG_PREC_FP64)
        k_energy_list<PREC_F64><<<NB_BLOCKS, NB_THREADS, 0, stream>>>(A, n, pbc, cut, d_nbr, d_nup, cap, nbp);
    else if (pbc.type != 0)
        return launch_pair_variant(pair_variant < 0 ? 0 : pair_variant, nbp);
    else
        k_energy_list<PREC_MIX><<<NB_BLOCKS, NB_THREADS, 0, stream>>>(A, n, pbc, cut, d_nbr, d_nup, cap, nbp);
    return NB_BLOCKS;
}

static const int kListVariants = 4;
static const int kGroupFirst = kListVariants + ClusterPairs::kVariants;   // first group-pair variant

int SingleEngine::pair_kernel_count() { return kGroupFirst + GroupPairs::kVariants; }

int SingleEngine::launch_pair_variant(int v, double* nbp) {
    if (v >= kGroupFirst)
        return grp.launch_energy(stream, v - kGroupFirst, d_fx, d_cls, ncls, group_geom(), nbp);
    if (v >= kListVariants) {
        launches += 1;   // the pack kernel in front of the cluster kernel
        return clp.launch_energy(stream, v - kListVariants, d_fx, d_prmf, cluster_geom(), nbp);
    }
    AtomsDev A = atoms();
    const double inv_f1 = cluster_geom().inv_f1;
    // the pruned rows when they are current (prepare_pair_kernel prunes before every launch that
    // needs it), else the Verlet rows
    const bool pr = prune_buf > 0.0 && !prune_dirty && d_prn;
    const int* rows = pr ? d_prn : d_nbr;
    const int* lens = pr ? d_pnup : d_nup;
    // cubic boxes: r^2 in fixed-point units scaled by the float-float square of the unit length
    const bool iso = A.Ls[0] == A.Ls[1] && A.Ls[1] == A.Ls[2] && A.Lsl[0] == A.Lsl[1] && A.Lsl[1] == A.Lsl[2];
    const double l2 = (double)A.Ls[0] + (double)A.Lsl[0];
    const double l2sq = l2 * l2;
    const float L2h = (float)l2sq, L2l = (float)(l2sq - (double)L2h);
    int blocks = 0;
#define MCG_LIST_MIX_ONE(U_, B_, ISO_, TY_)                                                                  \
    blocks = 152 * B_;                                                                                        \
    k_energy_list_mix<U_, B_, ISO_, TY_><<<152 * B_, NB_THREADS, TY_ ? sizeof(float4) * ncls : 0, stream>>>( \
        d_fx, d_prmf, d_cls, ncls, n, A.Ls[0], A.Ls[1], A.Ls[2], A.Lsl[0], A.Lsl[1], A.Lsl[2], L2h, L2l, cut, inv_f1, \
        rows, lens, cap, nbp);
#define MCG_LIST_MIX(U_, B_)                                                                                   \
    if (iso && ncls > 0) { MCG_LIST_MIX_ONE(U_, B_, true, true) }                                             \
    else if (iso) { MCG_LIST_MIX_ONE(U_, B_, true, false) }                                                   \
    else if (ncls > 0) { MCG_LIST_MIX_ONE(U_, B_, false, true) }                                              \
    else { MCG_LIST_MIX_ONE(U_, B_, false, false) }
    // grids sized to the residency each variant asks for (NB_THREADS threads per CTA)
    switch (v) {
    case 0: MCG_LIST_MIX(4, 4) break;
    case 1: MCG_LIST_MIX(5, 4) break;
    case 2: MCG_LIST_MIX(3, 5) break;
    default: MCG_LIST_MIX(6, 4) break;
    }
#undef MCG_LIST_MIX
#undef MCG_LIST_MIX_ONE
    return blocks;
}

// Times every pair-kernel variant on the current system (3 launches each) and keeps the fastest;
// the cluster-pair variants take part when the cluster list was built.
void SingleEngine::tune_pair_kernel() {
    cudaEvent_t a, b;
    pair_variant = 0;
    if (cudaEventCreate(&a) != cudaSuccess) return;
    if (cudaEventCreate(&b) != cudaSuccess) { cudaEventDestroy(a); return; }
    float best = 3.0e38f;
    const int nv = pair_kernel_count();
    int timed = 0;
    for (int v = 0; v < nv; v++) {
        if (v >= kListVariants && v < kGroupFirst && !clp.ok) continue;
        if (v >= kGroupFirst && !grp.ok) continue;
        timed++;
        launch_pair_variant(v, d_part);
        cudaEventRecord(a, stream);
        for (int r = 0; r < 3; r++) launch_pair_variant(v, d_part);
        cudaEventRecord(b, stream);
        float ms = 0.f;
        if (cudaEventSynchronize(b) != cudaSuccess || cudaEventElapsedTime(&ms, a, b) != cudaSuccess) continue;
        if (ms < best) { best = ms; pair_variant = v; }
    }
    launches += 4 * timed;
    cudaEventDestroy(a);
    cudaEventDestroy(b);
}

int SingleEngine::set_pair_kernel(int v) {
    if (v < -1 || v >= pair_kernel_count()) return fail(MCG_EINVAL, "pair-kernel variant out of range");
    if (v >= 0 && !uses_pair_variants())
        return fail(MCG_ENOTSUP, "pair-kernel variants apply to the mixed periodic switch energy");
    if (v >= kGroupFirst) {
        if (!grp_setup) return fail(MCG_ENOTSUP, "the group-pair kernels need the parameter-class table");
        int rc = ensure_pruned();
        if (!rc) rc = ensure_groups();
        if (rc) return rc;
        if (!grp.ok) return fail(MCG_ENOTSUP, "the group-pair rows could not be built for this system");
    } else if (v >= kListVariants) {
        int rc = ensure_clusters();
        if (rc) return rc;
        if (!clp.ok) return fail(MCG_ENOTSUP, "the cluster-pair list could not be built for this system");
    }
    pair_variant = v;
    return MCG_OK;
}

// The group-pair rows of the rows the per-atom list kernels read (pruned rows when pruning is on),
// rebuilt on first use after those rows changed.  A system whose group rows overflow the build's
// limits keeps the other kernels.
int SingleEngine::ensure_groups() {
    if (!grp_setup || !grp_dirty) return MCG_OK;
    grp_dirty = false;
    const bool pr = prune_buf > 0.0 && !prune_dirty && d_prn;
    const int grc = grp.build(stream, pr ? d_prn : d_nbr, pr ? d_pnup : d_nup, cap);
    launches += grp.build_launches;
    grp.build_launches = 0;
    if (grc == MCG_ECUDA) return grc;
    if (grc != MCG_OK) set_error("");
    return MCG_OK;
}

GroupGeom SingleEngine::group_geom() const {
    const ClusterGeom C = cluster_geom();
    GroupGeom G;
    for (int k = 0; k < 3; k++) { G.Ls[k] = C.Ls[k]; G.Ll[k] = C.Ll[k]; }
    G.iso = G.Ls[0] == G.Ls[1] && G.Ls[1] == G.Ls[2] && G.Ll[0] == G.Ll[1] && G.Ll[1] == G.Ll[2];
    const double l2 = (double)G.Ls[0] + (double)G.Ll[0];
    const double l2sq = l2 * l2;
    G.L2h = (float)l2sq;
    G.L2l = (float)(l2sq - (double)G.L2h);
    G.c2 = C.c2;
    G.n2 = C.n2;
    G.k3 = C.k3;
    G.inv_f1 = C.inv_f1;
    G.D = C.c2 - C.n2;
    G.inv_p1 = 1.0 / (double)((G.D * G.D) * std::fmaf(G.D, -2.0f, 3.0f * G.D));
    const double lmin = std::min(pbc.L[0], std::min(pbc.L[1], pbc.L[2]));
    G.emax = (float)(0.5 * lmin - std::sqrt((double)C.c2) - 1e-3);
    return G;
}

int SingleEngine::group_stats(int64_t* groups, int64_t* entries, int64_t* mask_pairs) {
    *groups = *entries = *mask_pairs = 0;
    if (!grp_setup) return MCG_OK;
    int rc = ensure_pruned();
    if (!rc) rc = ensure_groups();
    if (rc) return rc;
    if (grp.ok) { *groups = grp.ngroup; *entries = grp.nentries; *mask_pairs = grp.nbits; }
    return MCG_OK;
}

bool SingleEngine::uses_pair_variants() const {
    return hs.prec == MCG_PREC_MIXED && pbc.type != 0 && hs.cut == MCG_CUT_SWITCH;
}

// The cluster-pair form of the current Verlet list, built on first use after a list build (the
// tuner's first timing, a cluster variant chosen, or the statistics asked for).  A system whose
// clusters do not fit the build's shared-memory limits keeps the per-atom list kernels only.
int SingleEngine::ensure_clusters() {
    if (!clp_dirty) return MCG_OK;
    clp_dirty = false;
    const int crc = clp.build(stream, d_fx, n, hs.L, d_nbr, d_nup, d_nlo, cap);
    launches += clp.build_launches;
    clp.build_launches = 0;
    if (crc == MCG_OK) return ensure_part((size_t)2 * clp.ncl + 2 * 64 + 5 * 64 + 16);
    if (crc == MCG_ECUDA) return crc;
    set_error("");
    return MCG_OK;
}

// Before a launch of the mixed periodic switch energy: the first use times every variant (the
// cluster list built for it); a chosen cluster variant has its list brought up to date.  Runs
// before the caller takes the partial-sum buffer, which the cluster build may grow.
int SingleEngine::prepare_pair_kernel() {
    if (!uses_pair_variants()) return MCG_OK;
    int rc;
    if ((rc = ensure_pruned())) return rc;
    if (pair_variant < 0) {
        if ((rc = ensure_clusters())) return rc;
        if ((rc = ensure_groups())) return rc;
        tune_pair_kernel();
    }
    if (pair_variant >= kGroupFirst) {
        if ((rc = ensure_groups())) return rc;
        if (!grp.ok) pair_variant = 0;
    } else if (pair_variant >= kListVariants) {
        if ((rc = ensure_clusters())) return rc;
        if (!clp.ok) pair_variant = 0;
    }
    return MCG_OK;
}

// Prunes the Verlet rows for the pair kernel when they are stale: after a list build, a change of
// the buffer, or once an atom has moved more than half the buffer (less 1e-3 A) from its position
// at the last prune (host-side positions, minimum image).  The prune runs on the handle's stream
// between event records, so its device time can be read back without a synchronisation here.
int SingleEngine::ensure_pruned() {
    if (prune_buf <= 0.0 || !prune_dirty) return MCG_OK;
    int rc;
    if (prn_cap != cap) {   // the pruned rows share the Verlet rows' stride
        if (d_prn) cudaFree(d_prn);
        d_prn = nullptr;
        prn_cap = 0;
        if ((rc = dalloc(&d_prn, (size_t)n * cap))) return rc;
        prn_cap = cap;
    }
    if (!d_pnup && (rc = dalloc(&d_pnup, n))) return rc;
    if (!d_pkept && (rc = dalloc(&d_pkept, 1))) return rc;
    for (cudaEvent_t& e : ev_prune)
        if (!e) CK(cudaEventCreate(&e));
    const AtomsDev A = atoms();
    const double rp = hs.rc + prune_buf;
    const float rp2 = (float)(rp * rp * (1.0 + 1e-5));   // above any FP32 rounding of r^2
    CK(cudaMemsetAsync(d_pkept, 0, sizeof(unsigned long long), stream));
    CK(cudaEventRecord(ev_prune[0], stream));
    k_prune_rows<<<NB_BLOCKS, NB_THREADS, 0, stream>>>(d_fx, n, A.Ls[0], A.Ls[1], A.Ls[2], A.Lsl[0], A.Lsl[1], A.Lsl[2],
                                                       rp2, d_nbr, d_nup, cap, d_prn, d_pnup, d_pkept);
    CK(cudaGetLastError());
    CK(cudaEventRecord(ev_prune[1], stream));
    prune_x = host_x;
    prune_y = host_y;
    prune_z = host_z;
    const double lim = std::max(0.0, 0.5 * prune_buf - 1e-3);
    prune_lim2 = lim * lim;
    prune_dirty = false;
    grp_dirty = grp_setup;    // the group rows follow the pruned rows
    prunes++;
    launches += 1;
    return MCG_OK;
}

// An atom's coordinates changed on the host side: the pruned rows go stale once it is further
// than the limit from where it was at the last prune.
void SingleEngine::note_moved(int a) {
    double d2 = 0.0;
    const double p[3] = {host_x[a] - prune_x[a], host_y[a] - prune_y[a], host_z[a] - prune_z[a]};
    for (int k = 0; k < 3; k++) {
        const double d = p[k] - hs.L[k] * std::nearbyint(p[k] / hs.L[k]);
        d2 += d * d;
    }
    if (!(d2 <= prune_lim2)) prune_dirty = true;
}

int SingleEngine::set_prune_buffer(double buffer) {
    if (!(buffer >= 0.0) || !std::isfinite(buffer)) return fail(MCG_EINVAL, "prune buffer must be finite and >= 0");
    if (buffer > 0.0 && !uses_pair_variants())
        return fail(MCG_ENOTSUP, "pruning applies to the mixed periodic switch energy");
    prune_buf = buffer;
    prune_dirty = true;
    grp_dirty = grp_setup;
    return MCG_OK;
}

int SingleEngine::prune_stats(int64_t* entries, int64_t* nprunes, float* last_ms) {
    *entries = 0;
    *nprunes = prunes;
    *last_ms = 0.f;
    if (prunes == 0 || !d_pkept) return MCG_OK;
    unsigned long long k = 0;
    CK(cudaMemcpyAsync(&k, d_pkept, sizeof(k), cudaMemcpyDeviceToHost, stream));
    CK(cudaStreamSynchronize(stream));
    CK(cudaEventElapsedTime(last_ms, ev_prune[0], ev_prune[1]));
    *entries = (int64_t)k;
    return MCG_OK;
}

int SingleEngine::cluster_stats(int64_t* clusters, int64_t* cluster_pairs, int64_t* mask_pairs) {
    *clusters = *cluster_pairs = *mask_pairs = 0;
    if (!uses_pair_variants()) return MCG_OK;
    int rc = ensure_clusters();
    if (rc) return rc;
    if (clp.ok) { *clusters = clp.ncl; *cluster_pairs = clp.npairs; *mask_pairs = clp.nbits; }
    return MCG_OK;
}

ClusterGeom SingleEngine::cluster_geom() const {
    ClusterGeom G;
    AtomsDev A = atoms();
    for (int k = 0; k < 3; k++) {
        G.Ls[k] = A.Ls[k];
        G.Ll[k] = A.Lsl[k];
        G.Lf[k] = (float)hs.L[k];
        G.iLf[k] = (float)(1.0 / hs.L[k]);
        G.lim[k] = (float)(hs.L[k] - hs.rc - 0.01);
    }
    G.c2 = cut.c2f;
    G.n2 = cut.n2f;
    G.k3 = cut.c2f - 3.0f * cut.n2f;
    const float pr = (float)(hs.rc + 0.01);
    G.prune2 = pr * pr;
    // the FP32 switch polynomial at u = ron^2, as the kernel forms it
    const float a = G.c2 - G.n2;
    const float aa = a * a;
    const float bb = std::fmaf(2.0f, G.n2, G.k3);
    const float f1 = aa * bb;
    G.inv_f1 = 1.0 / (double)f1;
    return G;
}

int SingleEngine::ensure_part(size_t count) {
    if (count <= part_cap) return MCG_OK;
    if (d_part) cudaFree(d_part);
    d_part = nullptr;
    part_cap = 0;
    int rc = dalloc(&d_part, count);
    if (rc) return rc;
    part_cap = count;
    return MCG_OK;
}

int SingleEngine::time_nonbonded(int reps, float* ms) {
    if (hs.cut != MCG_CUT_SWITCH) return fail(MCG_ENOTSUP, "the pair-kernel timing covers the switch mode");
    {
        int rc = prepare_pair_kernel();
        if (rc) return rc;
    }
    cudaEvent_t a, b;
    CK(cudaEventCreate(&a));
    CK(cudaEventCreate(&b));
    launch_nonbonded(d_part);                       // warm
    CK(cudaEventRecord(a, stream));
    for (int r = 0; r < reps; r++) launch_nonbonded(d_part);
    CK(cudaEventRecord(b, stream));
    CK(cudaEventSynchronize(b));
    CK(cudaEventElapsedTime(ms, a, b));
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    launches += reps + 1;
    return MCG_OK;
}

int SingleEngine::time_nonbonded_flushed(int reps, float* ms) {
    if (hs.cut != MCG_CUT_SWITCH) return fail(MCG_ENOTSUP, "the pair-kernel timing covers the switch mode");
    {
        int rc = prepare_pair_kernel();
        if (rc) return rc;
    }
    constexpr size_t kFlush = (size_t)256 << 20;   // twice the L2
    unsigned char* junk = nullptr;
    CK(cudaMalloc(&junk, kFlush));
    cudaEvent_t a, b;
    if (cudaEventCreate(&a) != cudaSuccess) { cudaFree(junk); return fail(MCG_ECUDA, "cudaEventCreate"); }
    if (cudaEventCreate(&b) != cudaSuccess) { cudaEventDestroy(a); cudaFree(junk); return fail(MCG_ECUDA, "cudaEventCreate"); }
    float total = 0.0f;
    cudaError_t e = cudaSuccess;
    for (int r = 0; r < reps && e == cudaSuccess; r++) {
        e = cudaMemsetAsync(junk, r & 0xff, kFlush, stream);
        if (e == cudaSuccess) e = cudaEventRecord(a, stream);
        if (e == cudaSuccess) launch_nonbonded(d_part);
        if (e == cudaSuccess) e = cudaEventRecord(b, stream);
        if (e == cudaSuccess) e = cudaEventSynchronize(b);
        float t = 0.0f;
        if (e == cudaSuccess) e = cudaEventElapsedTime(&t, a, b);
        total += t;
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    cudaFree(junk);
    if (e != cudaSuccess) return fail(MCG_ECUDA, std::string("flushed pair-kernel timing: ") + cudaGetErrorString(e));
    launches += reps;
    *ms = total;
    return MCG_OK;
}

AtomsDev SingleEngine::atoms() const {
    AtomsDev A;
    A.pq = d_pq; A.es = d_es; A.es14 = d_es14; A.fx = d_fx; A.esf = d_esf; A.esf14 = d_esf14; A.qf = d_qf;
    for (int k = 0; k < 3; k++) {
        const double ls = hs.L[k] / 4294967296.0;
        A.Ls[k] = (float)ls;
        A.Lsl[k] = (float)(ls - (double)A.Ls[k]);
    }
    return A;
}

BondedDev SingleEngine::bonded() const {
    return BondedDev{d_bonds, (int)hs.bonds.size(), d_ubs, (int)hs.ubs.size(), d_angles, (int)hs.angles.size(),
                     d_dihes, (int)hs.dihes.size(), d_imprs, (int)hs.imprs.size()};
}

int SingleEngine::build_list() {
    const double rl = hs.rc + hs.dcut;
    Grid g;
    g.periodic = hs.pbc != MCG_PBC_NONE;
    double ext[3];
    if (g.periodic) {
        for (int k = 0; k < 3; k++) { ext[k] = hs.L[k]; g.lo[k] = 0; g.inv[k] = 0; }
    } else {
        for (int k = 0; k < 3; k++) {
            const std::vector<double>& c = k == 0 ? host_x : (k == 1 ? host_y : host_z);
            double lo = *std::min_element(c.begin(), c.end()), hi = *std::max_element(c.begin(), c.end());
            ext[k] = std::max(hi - lo, 1e-6);
            g.lo[k] = lo;
            g.inv[k] = 1.0 / ext[k] * (1.0 - 1e-12);
        }
    }
    for (int k = 0; k < 3; k++) g.nc[k] = std::max(1, (int)std::floor(2.0 * ext[k] / rl));
    while ((long long)g.nc[0] * g.nc[1] * g.nc[2] > (1 << 20))
        for (int k = 0; k < 3; k++) g.nc[k] = std::max(1, g.nc[k] / 2);
    for (int k = 0; k < 3; k++) g.csf[k] = (float)(ext[k] / g.nc[k] * (1.0 - 1e-6));
    int ncell = g.nc[0] * g.nc[1] * g.nc[2];
    int rc;
    if (ncell > ncell_cap) {
        if (d_cell_count) { cudaFree(d_cell_count); cudaFree(d_cell_start); cudaFree(d_cell_fill); }
        if ((rc = dalloc(&d_cell_count, ncell)) || (rc = dalloc(&d_cell_start, ncell + 1)) || (rc = dalloc(&d_cell_fill, ncell)))
            return rc;
        ncell_cap = ncell;
    }
    if (!d_cell_of) {
        if ((rc = dalloc(&d_cell_of, n)) || (rc = dalloc(&d_cell_atoms, n)) || (rc = dalloc(&d_nup, n)) || (rc = dalloc(&d_nlo, n)))
            return rc;
    }
    if (cap == 0) {
        // initial capacity from the density of the list sphere, grown on overflow below
        double vol = g.periodic ? hs.L[0] * hs.L[1] * hs.L[2] : 0.0;
        double est = g.periodic ? (4.0 / 3.0 * PI * rl * rl * rl) * n / vol : n;
        cap = (int)std::min<double>(n, est * 1.3 + 64);
        cap = (cap + 31) & ~31;
        if ((rc = dalloc(&d_nbr, (size_t)n * cap))) return rc;
    }
    ListParams lp{rl * rl, cap, hs.maxExclSpan, {0, 0, 0}, {0, 0, 0}, 0.f, 0.f, 0.f};
    {
        double t = hs.rc + hs.dcut;  // (cutoff + deltacut)^2 as List_nonBonded.cpp:842-843
        lp.cutnb2 = t * t;
        const AtomsDev A = atoms();
        for (int k = 0; k < 3; k++) { lp.Ls[k] = A.Ls[k]; lp.Ll[k] = A.Lsl[k]; }
        lp.lo2 = (float)(lp.cutnb2 * (1.0 - 1e-4));
        lp.hi2 = (float)(lp.cutnb2 * (1.0 + 1e-4));
        lp.reach2 = (float)(lp.cutnb2 * (1.0 + 1e-5) + 1e-2);
    }
    for (int attempt = 0; attempt < 3; attempt++) {
        CK(cudaMemsetAsync(d_cell_count, 0, sizeof(int) * ncell, stream));
        CK(cudaMemsetAsync(d_maxrow, 0, sizeof(int), stream));
        k_cell_assign<<<(n + 255) / 256, 256, 0, stream>>>(d_pq, n, pbc, g, d_cell_of, d_cell_count);
        k_cell_scan<<<1, 1024, 0, stream>>>(d_cell_count, ncell, d_cell_start, d_cell_fill);
        k_cell_scatter<<<(n + 255) / 256, 256, 0, stream>>>(d_cell_of, n, d_cell_start, d_cell_fill, d_cell_atoms);
        k_cell_sort<<<ncell, 256, 0, stream>>>(d_cell_start, ncell, d_cell_atoms);
        int blocks = std::min((n + 7) / 8, NB_BLOCKS * 2);
        k_build_rows<<<blocks, 256, 0, stream>>>(d_pq, d_fx, d_frozen, n, pbc, g, lp, d_cell_of, d_cell_start, d_cell_atoms,
                                                 d_xs, d_xd, d_nbr, d_nup, d_nlo, d_maxrow);
        CK(cudaGetLastError());
        int maxrow = 0;
        CK(cudaMemcpyAsync(&maxrow, d_maxrow, sizeof(int), cudaMemcpyDeviceToHost, stream));
        CK(cudaStreamSynchronize(stream));
        last_max_row = maxrow;
        if (maxrow <= cap) {
            clp_dirty = uses_pair_variants();   // the cluster form follows on first use
            prune_dirty = true;                 // and so do the pruned rows
            grp_dirty = grp_setup;              // and the group rows
            return MCG_OK;
        }
        cudaFree(d_nbr);
        d_nbr = nullptr;
        cap = ((int)(maxrow * 1.1) + 32 + 31) & ~31;
        lp.cap = cap;
        if ((rc = dalloc(&d_nbr, (size_t)n * cap))) return rc;
    }
    return fail(MCG_ECAPACITY, "Verlet row capacity could not be grown");
}

int SingleEngine::energy(double ener[10]) {
    if (hs.cut == MCG_CUT_SWITCH) {
        int rc = prepare_pair_kernel();
        if (rc) return rc;
    }
    AtomsDev A = atoms();
    double* nbp = d_part;
    int nnb = 0;
    if (hs.cut == MCG_CUT_SWITCH) {
        nnb = launch_nonbonded(nbp);
    } else {
        nnb = ntile * (ntile + 1) / 2;
        if (hs.prec == MCG_PREC_FP64)
            k_energy_all<PREC_F64><<<nnb, TILE, 0, stream>>>(A, n, pbc, cut, d_fxs, d_fxd, ntile, nbp);
        else
            k_energy_all<PREC_MIX><<<nnb, TILE, 0, stream>>>(A, n, pbc, cut, d_fxs, d_fxd, ntile, nbp);
    }
    double* p14 = nbp + 2 * (size_t)nnb;
    int n14b = 0;
    if (n14 > 0) {
        n14b = std::min(64, (n14 + 255) / 256);
        if (hs.prec == MCG_PREC_FP64) k_energy_14<PREC_F64><<<n14b, 256, 0, stream>>>(A, pbc, cut, d_p14, n14, p14);
        else k_energy_14<PREC_MIX><<<n14b, 256, 0, stream>>>(A, pbc, cut, d_p14, n14, p14);
    }
    double* bd = p14 + 2 * (size_t)n14b;
    BondedDev B = bonded();
    int nterm = B.nb + B.na + B.nu + B.nd + B.ni;
    int nbd = 0;
    if (nterm > 0) {
        nbd = std::min(64, (nterm + 255) / 256);
        k_bonded<<<nbd, 256, 0, stream>>>(B, pbc, d_pq, bd);
    }
    k_finalize<<<1, 256, 0, stream>>>(nbp, nnb, p14, n14b, bd, nbd, d_map + 8);
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(stream));
    for (int k = 0; k < 10; k++) ener[k] = ((volatile double*)h_map)[8 + k];
    launches += 1 + (n14b > 0) + (nbd > 0) + 1;
    return MCG_OK;
}

int SingleEngine::set_coords(const double* x, const double* y, const double* z) {
    std::vector<double4_32a> pq(n);
    for (int i = 0; i < n; i++) {
        if (!std::isfinite(x[i]) || !std::isfinite(y[i]) || !std::isfinite(z[i]))
            return fail(MCG_EINVAL, "non-finite coordinate at atom " + std::to_string(i));
        pq[i] = make_double4_32a(x[i], y[i], z[i], hs.q[i]);
        host_x[i] = x[i]; host_y[i] = y[i]; host_z[i] = z[i];
    }
    if (!prune_dirty)
        for (int i = 0; i < n && !prune_dirty; i++) note_moved(i);
    CK(cudaMemcpyAsync(d_pq, pq.data(), sizeof(double4_32a) * n, cudaMemcpyHostToDevice, stream));
    k_fix_all<<<(n + 255) / 256, 256, 0, stream>>>(n, d_pq, d_cls_of, d_fx, pbc);
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(stream));
    return MCG_OK;
}

int SingleEngine::get_coords(double* x, double* y, double* z) {
    std::vector<double4_32a> pq(n);
    CK(cudaMemcpyAsync(pq.data(), d_pq, sizeof(double4_32a) * n, cudaMemcpyDeviceToHost, stream));
    CK(cudaStreamSynchronize(stream));
    for (int i = 0; i < n; i++) { x[i] = pq[i].x; y[i] = pq[i].y; z[i] = pq[i].z; }
    return MCG_OK;
}

int SingleEngine::delta_e(int m, const int* atoms_in, const double* nx, const double* ny, const double* nz, double* de) {
    pending_m = 0;   // a new proposal replaces the pending one, also when it is rejected
    if (m <= 0 || m > MAX_MOVED) return fail(MCG_EINVAL, "moved-set size must be in [1, 1024]");
    // sort the moved set (keeps proposal coordinates paired), reject duplicates
    std::vector<int> ord(m);
    std::iota(ord.begin(), ord.end(), 0);
    std::sort(ord.begin(), ord.end(), [&](int a, int b) { return atoms_in[a] < atoms_in[b]; });
    // staged as [idx: m ints | xyz: 3m doubles | terms: 2 ints each], packed so that one small
    // copy carries the proposal; the device copy stays in place for commit()
    const size_t off_xyz = ((size_t)4 * m + 15) & ~(size_t)15, off_terms = off_xyz + (size_t)24 * m;
    char* st = (char*)h_stage;
    int* idx = (int*)st;
    double* xyz = (double*)(st + off_xyz);
    int* terms = (int*)(st + off_terms);
    for (int k = 0; k < m; k++) {
        int a = atoms_in[ord[k]];
        if (a < 0 || a >= n) return fail(MCG_EINVAL, "moved atom index out of range");
        if (k > 0 && a == idx[k - 1]) return fail(MCG_EINVAL, "duplicate moved atom");
        double px = nx[ord[k]], py = ny[ord[k]], pz = nz[ord[k]];
        if (!std::isfinite(px) || !std::isfinite(py) || !std::isfinite(pz)) return fail(MCG_EINVAL, "non-finite proposal");
        idx[k] = a;
        xyz[3 * k] = px; xyz[3 * k + 1] = py; xyz[3 * k + 2] = pz;
    }
    // bonded terms touching the moved set, each once
    stamp++;
    int nt = 0;
    const size_t tcap = (stage_bytes - 64 - off_terms) / 8;   // the last 64 bytes take de back
    for (int k = 0; k < m; k++) {
        int a = idx[k];
        for (int t = term_start[a]; t < term_start[a + 1]; t++) {
            int kind = term_data[2 * t], ti = term_data[2 * t + 1];
            size_t gk = (size_t)ti * 5 + kind;
            if (gk >= term_seen.size()) term_seen.resize(gk + 1, 0);
            if (term_seen[gk] == stamp) continue;
            term_seen[gk] = stamp;
            if ((size_t)nt >= tcap) return fail(MCG_ECAPACITY, "too many bonded terms in one move");
            terms[2 * nt] = kind; terms[2 * nt + 1] = ti;
            nt++;
        }
    }
    MoveDev mv;
    mv.m = m;
    mv.idx = (const int*)d_stage;
    mv.xyz = (const double*)((char*)d_stage + off_xyz);
    mv.terms = (const int*)((char*)d_stage + off_terms);
    mv.nterms = nt;
    MoveInline inl;
    inl.m = 0; inl.nterms = 0;
    if (m <= INL_M && nt <= INL_T) {
        inl.m = m; inl.nterms = nt;
        memcpy(inl.idx, idx, 4 * (size_t)m);
        memcpy(inl.xyz, xyz, 24 * (size_t)m);
        memcpy(inl.terms, terms, 8 * (size_t)nt);
    } else {
        CK(cudaMemcpyAsync(d_stage, h_stage, off_terms + (size_t)nt * 8, cudaMemcpyHostToDevice, stream));
    }
    AtomsDev A = atoms();
    BondedDev B = bonded();
    // slices per moved atom: about one partner per thread for a Verlet row (64 threads), about
    // four per thread over all atoms in full mode (256 threads), at most two blocks per SM in all
    const bool sw = hs.cut == MCG_CUT_SWITCH;
    const int threads = sw ? 64 : 256;
    const int span = sw ? cap : n;
    int S = (span + (sw ? 64 : 1024) - 1) / (sw ? 64 : 1024);
    S = std::max(1, std::min(S, std::max(1, 304 / m)));
    S = std::min(S, std::max(1, MAX_MOVED / m));   // m*S + 1 partials fit the scratch
    if (hs.prec == MCG_PREC_FP64)
        k_delta_e<PREC_F64><<<m * S + 1, threads, 0, stream>>>(A, n, pbc, cut, mv, d_nbr, d_nup, d_nlo, cap, d_fxs,
                                                                d_fxd, d_c14s, d_c14d, B, S, d_part, d_ticket, d_map, inl);
    else
        k_delta_e<PREC_MIX><<<m * S + 1, threads, 0, stream>>>(A, n, pbc, cut, mv, d_nbr, d_nup, d_nlo, cap, d_fxs,
                                                                d_fxd, d_c14s, d_c14d, B, S, d_part, d_ticket, d_map, inl);
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(stream));   // de lands in mapped host memory
    *de = ((volatile double*)h_map)[0];
    pending_m = m;
    pending_inline = inl.m > 0;
    pending_off_xyz = off_xyz;
    pending_idx.assign(idx, idx + m);
    pending_xyz.assign(xyz, xyz + 3 * m);
    launches += 1;
    return MCG_OK;
}

// ---- device-resident Metropolis run (MC_metropolis::run, src/MC_metropolis.cpp:80-165) ---------
// For translation moves of atom sets without bonded terms in a periodic switched system, with no
// per-step output: the whole step runs on the device, a launch covering the steps up to the next
// list update (MC_metropolis.cpp:151).  The random numbers are the reference's: the raw 32-bit words of
// the host's std::mt19937, turned into doubles as libstdc++'s generate_canonical<double, 53> does
// (two words, w0 + w1 2^32 rounded once, times 2^-64; a result of 1 becomes the largest double
// below 1) and into uniform_real_distribution values as (b - a) u + a, every operation rounded on
// its own as the reference's uncontracted host code rounds it.
constexpr int RP_MAXT = SingleEngine::kReplayMaxTypes;   // move types
constexpr int RP_MAXM = SingleEngine::kReplayMaxAtoms;   // atoms of one move

bool SingleEngine::replay_fits(const std::vector<MoveKind>& moves) {
    if (moves.empty() || (int)moves.size() > RP_MAXT) return false;
    for (const MoveKind& mk : moves)
        for (int k = 0; k < mk.ninst(); k++) {
            int m = 0;
            for (int r = mk.rstart[k]; r < mk.rstart[k + 1]; r++) m += mk.ranges[2 * r + 1] - mk.ranges[2 * r] + 1;
            if (m > RP_MAXM) return false;
        }
    return true;
}
struct ReplayTables {
    int nmvtyp;
    int ninst[RP_MAXT];           // instances of each move type
    int ibase[RP_MAXT];           // first global instance of each type
    int each[RP_MAXT];            // dmax adjustment period (0: never), MC::adjust_dmax (MC.cpp:165-173)
    double target[RP_MAXT];       // target acceptance, percent
    const int* inst_first;        // per global instance: its first (first, last) atom range; one past the end last
    const int* ranges;            // (first, last) atom pairs
    int ninst_all, nranges;       // sizes of the two (instances + 1 entries, nranges pairs)
};
struct ReplayState {
    double etot;
    long long acc;
    long long cursor;             // random words consumed from the launch's buffer
    int steps_done;               // the last step completed
    int status;                   // 0 ok; 1 out of random words (resume after steps_done); 2 move too large
    double dmax[RP_MAXT];
    int acc_tmp[RP_MAXT];
};

__device__ __forceinline__ double rp_canonical(const uint32_t* __restrict__ w, long long& cur) {
    const double sum = __dadd_rn((double)w[cur], __dmul_rn((double)w[cur + 1], 4294967296.0));
    cur += 2;
    const double r = __dmul_rn(sum, 5.421010862427522170037264e-20);   // 2^-64
    return r >= 1.0 ? 0.99999999999999988898 : r;                       // nextafter(1, 0)
}

// Tools::rint wrap of one coordinate (PerConditions::applyPBC, PerConditions.cpp:244-285)
__device__ __forceinline__ double rp_wrap(double v, double L, double rL) {
    const double t = __dmul_rn(rL, v);
    const double r = (double)(t >= 0.0 ? __double2int_rz(__dadd_rn(t, 0.5)) : __double2int_rz(__dsub_rn(t, 0.5)));
    return __dsub_rn(v, __dmul_rn(L, r));
}

// One thread-block cluster of RP_CL CTAs of RP_NT threads runs the steps.  On GB300 a warp's FP64
// instruction holds its scheduler's narrow FP64 pipe for tens of cycles whatever its active lanes,
// so a step costs about (warps per scheduler) x (the dependent FP64 operations of one thread):
//  - the proposal's uniforms (move type, instance and RP_TRIES unit-ball tries at once) are formed
//    by the lanes of warp 0 in one pass, and the first accepted try is picked by ballot;
//  - the dE terms are spread one per thread over the cluster's schedulers (CTAs first, then warps,
//    then lanes), the old and the new energy of a pair on different threads;
//  - each CTA's partial sums go to every CTA's shared memory, so every CTA sums them in rank order
//    and takes the same decision; CTA 0 commits, and a cluster barrier orders the commit before
//    the next step's reads.
// The launch's random words, and the move-instance tables when they fit, are copied into each
// CTA's shared memory first: the proposal's loads are then shared-memory loads, not L2 round trips.
// While the four warps of a CTA take the dE terms, a fifth forms the next step's uniforms: the next
// step's words start at this step's post-proposal cursor, or 2 words later when this step draws an
// acceptance uniform, so 27 uniforms from that cursor cover both cases; the warp forms both cases'
// move type, instance and RP_TRIES unit-ball tries.  The next proposal picks the case its cursor
// matches and only scales, orders and wraps; when none of those tries lies in the ball it goes on
// with the following ones as before.  The same operations on the same words: the same proposals.
// Measured on the 864-atom argon box (moves per second, host work included): 49.8k with one
// 256-thread CTA (its ~200 dE terms at two warps per scheduler), 89.9k with the cluster and the
// words read from global memory, 94.8k with them in shared memory, 99.9k with the fifth warp.
constexpr int RP_CL = 8;
constexpr int RP_NT = 128;
constexpr int RP_TRIES = 8;
constexpr int RP_SPEC = 32;            // a fifth warp: the next step's uniforms, formed during this step's dE
constexpr int RP_WORDS = 8192;        // random words of one launch, staged in each CTA's shared memory
constexpr int RP_TAB = 3072;          // ints of the instance tables staged with them when they fit

__device__ __forceinline__ double rp_canonical_at(const uint32_t* __restrict__ w, long long at) {
    long long cur = at;
    return rp_canonical(w, cur);
}

__global__ void __cluster_dims__(RP_CL, 1, 1) __launch_bounds__(RP_NT + RP_SPEC)
    k_replay(AtomsDev A, double4_32a* pq, uint4* fx, PbcDev pbc, CutDev cut, const int* __restrict__ nbr,
             const int* __restrict__ nup, const int* __restrict__ nlo, int cap, const int* __restrict__ c14s,
             const int* __restrict__ c14d, ReplayTables T, const uint32_t* __restrict__ words, long long nwords,
             ReplayState* st, int s0, int s1, double beta) {
    namespace cg = cooperative_groups;
    cg::cluster_group cluster = cg::this_cluster();
    __shared__ ReplayState S;
    __shared__ int s_idx[RP_MAXM];
    __shared__ double s_xyz[3 * RP_MAXM];
    __shared__ double s_r[3];
    __shared__ int s_m, s_type, s_stop, s_acc;
    __shared__ long long s_cur;
    __shared__ double s_part[2][RP_NT / 32];
    __shared__ double2 s_cl[RP_CL];
    __shared__ __align__(16) uint32_t s_words[RP_WORDS];
    __shared__ int s_tab[RP_TAB];
    // the next step's uniforms, both cases (0: no acceptance draw in this step, 1: one)
    __shared__ double s_sx[2 * RP_TRIES], s_sy[2 * RP_TRIES], s_sz[2 * RP_TRIES], s_sq[2 * RP_TRIES];
    __shared__ int s_st[2], s_sg[2], s_sok;
    __shared__ long long s_sbase;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    constexpr int NW = RP_NT / 32, G = RP_CL * RP_NT;
    for (int i = tid; i < (int)(nwords >> 2); i += blockDim.x)
        reinterpret_cast<uint4*>(s_words)[i] = reinterpret_cast<const uint4*>(words)[i];
    const bool tab_sh = T.ninst_all + 2 * T.nranges <= RP_TAB;
    if (tab_sh) {
        for (int i = tid; i < T.ninst_all; i += blockDim.x) s_tab[i] = T.inst_first[i];
        for (int i = tid; i < 2 * T.nranges; i += blockDim.x) s_tab[T.ninst_all + i] = T.ranges[i];
    }
    if (tid == 0) s_sok = 0;
    const int* inst_first = tab_sh ? s_tab : T.inst_first;
    const int* ranges = tab_sh ? s_tab + T.ninst_all : T.ranges;
    const int rank = (int)cluster.block_rank();
    const int gslot = rank + RP_CL * (warp + NW * lane);   // this thread's place in the spread order
    if (tid == 0) S = *st;
    cluster.sync();   // every CTA of the cluster is running before any writes into its shared memory
    for (int step = s0 + 1; step <= s1; step++) {
        if (warp == 0) {
            // the proposal (MC.cpp:142-156): type and instance from the words at cur and cur + 2,
            // unit-ball tries of 3 uniforms each from cur + 4 on (6 words a try), RP_TRIES at a time
            const long long cur = S.cursor;
            bool out = cur + 256 > nwords;
            int t = 0, m = 0, first = -1;
            int sv = -1;   // the case of the uniforms formed during the previous step that matches cur
            if (!out && s_sok) sv = cur == s_sbase ? 0 : (cur == s_sbase + 2 ? 1 : -1);
            if (!out) {
                int g;
                if (sv >= 0) {
                    t = s_st[sv];
                    g = s_sg[sv];
                } else {
                    double u = 0.0;
                    if (lane < 2) u = rp_canonical_at(s_words, cur + 2 * lane);
                    const double u0 = __shfl_sync(0xffffffffu, u, 0), u1 = __shfl_sync(0xffffffffu, u, 1);
                    t = (int)__dmul_rn((double)T.nmvtyp, u0);
                    g = T.ibase[t] + (int)__dmul_rn((double)T.ninst[t], u1);
                }
                if (lane == 0) {
                    for (int r = inst_first[g]; r < inst_first[g + 1]; r++)
                        for (int a = ranges[2 * r]; a <= ranges[2 * r + 1]; a++) {
                            if (m < RP_MAXM) s_idx[m] = a;
                            m++;
                        }
                }
                m = __shfl_sync(0xffffffffu, m, 0);
                int pass0 = 0;
                if (sv >= 0) {   // the first RP_TRIES tries, formed in advance
                    const unsigned ok = __ballot_sync(0xffffffffu, lane < RP_TRIES && s_sq[sv * RP_TRIES + lane] <= 1.0);
                    if (ok) {
                        const int k = __ffs(ok) - 1;
                        first = k;
                        if (lane == k) {
                            const double dm = S.dmax[t];
                            const int e = sv * RP_TRIES + k;
                            s_r[0] = __dmul_rn(s_sx[e], dm); s_r[1] = __dmul_rn(s_sy[e], dm); s_r[2] = __dmul_rn(s_sz[e], dm);
                        }
                    }
                    pass0 = 1;
                }
                for (int pass = pass0; first < 0; pass++) {
                    const long long cb = cur + 4 + 6LL * RP_TRIES * pass;
                    if (cb + 6LL * RP_TRIES + 2 > nwords) { out = true; break; }   // the pass and the acceptance draw
                    double v = 0.0;
                    if (lane < 3 * RP_TRIES) v = __dadd_rn(__dmul_rn(rp_canonical_at(s_words, cb + 2 * lane), 2.0), -1.0);
                    const double x = __shfl_sync(0xffffffffu, v, (3 * lane) & 31);
                    const double y = __shfl_sync(0xffffffffu, v, (3 * lane + 1) & 31);
                    const double z = __shfl_sync(0xffffffffu, v, (3 * lane + 2) & 31);
                    const double q = __dadd_rn(__dadd_rn(__dmul_rn(x, x), __dmul_rn(y, y)), __dmul_rn(z, z));
                    const unsigned ok = __ballot_sync(0xffffffffu, lane < RP_TRIES && q <= 1.0);
                    if (ok) {
                        const int k = __ffs(ok) - 1;
                        first = pass * RP_TRIES + k;
                        if (lane == k) {
                            const double dm = S.dmax[t];
                            s_r[0] = __dmul_rn(x, dm); s_r[1] = __dmul_rn(y, dm); s_r[2] = __dmul_rn(z, dm);
                        }
                    }
                }
            }
            if (lane == 0) {
                s_stop = 0;
                if (out) { s_stop = 1; S.status = 1; }
                else if (m > RP_MAXM) { s_stop = 1; S.status = 2; }
                else {
                    for (int i = 1; i < m; i++) {        // ascending atom order (the partner lookup bisects)
                        const int v = s_idx[i];
                        int k = i - 1;
                        while (k >= 0 && s_idx[k] > v) { s_idx[k + 1] = s_idx[k]; k--; }
                        s_idx[k + 1] = v;
                    }
                    s_m = m;
                    s_type = t;
                    s_cur = cur + 4 + 6LL * (first + 1);
                }
            }
            __syncwarp();
            if (!out && m <= RP_MAXM)
                for (int i = lane; i < 3 * m; i += 32) {   // the moved atoms' new positions, wrapped
                    const int k = i / 3, c = i - 3 * k;
                    const double4_32a p = pq[s_idx[k]];
                    const double pc = c == 0 ? p.x : (c == 1 ? p.y : p.z);
                    s_xyz[i] = rp_wrap(__dadd_rn(pc, s_r[c]), pbc.L[c], pbc.rL[c]);
                }
        }
        __syncthreads();
        if (s_stop) break;   // the same in every CTA: each formed the same proposal from the same words
        if (warp == NW) {
            // the next step's uniforms (words from b = this step's post-proposal cursor): type and
            // instance of case v from uniforms v and v + 1, try k from v + 2 + 3k .. v + 4 + 3k
            const long long b = s_cur;
            const bool ok = b + 54 <= nwords;
            double c = 0.0;
            if (ok && lane < 27) c = rp_canonical_at(s_words, b + 2 * lane);
            const double cn = __shfl_sync(0xffffffffu, c, (lane + 1) & 31);
            if (lane < 2) {
                const int tv = (int)__dmul_rn((double)T.nmvtyp, c);
                s_st[lane] = tv;
                s_sg[lane] = T.ibase[tv] + (int)__dmul_rn((double)T.ninst[tv], cn);
            }
            const int i0 = (lane >> 3) + 2 + 3 * (lane & 7);
            const double cx = __shfl_sync(0xffffffffu, c, i0 & 31), cy = __shfl_sync(0xffffffffu, c, (i0 + 1) & 31),
                         cz = __shfl_sync(0xffffffffu, c, (i0 + 2) & 31);
            if (lane < 2 * RP_TRIES) {
                const double x = __dadd_rn(__dmul_rn(cx, 2.0), -1.0), y = __dadd_rn(__dmul_rn(cy, 2.0), -1.0),
                             z = __dadd_rn(__dmul_rn(cz, 2.0), -1.0);
                s_sx[lane] = x; s_sy[lane] = y; s_sz[lane] = z;
                s_sq[lane] = __dadd_rn(__dadd_rn(__dmul_rn(x, x), __dmul_rn(y, y)), __dmul_rn(z, z));
            }
            if (lane == 0) { s_sbase = b; s_sok = ok ? 1 : 0; }
        }
        // dE of the moved set over its Verlet partners and 1-4 pairs, FP64 (as k_delta_e): term
        // (k, t, side) of the moved atoms' partner lists, numbered in list order, goes to the thread
        // whose gslot it equals modulo G; side 0 is the old pair energy (subtracted), 1 the new
        const int m = s_m;
        auto slot = [&](int j) -> int {
            int lo = 0, hi = m - 1;
            while (lo <= hi) {
                const int mid = (lo + hi) >> 1, v = s_idx[mid];
                if (v == j) return mid;
                if (v < j) lo = mid + 1; else hi = mid - 1;
            }
            return -1;
        };
        double del = 0.0, dvd = 0.0;
        const uint4 f0 = make_uint4(0, 0, 0, 0);
        int base = 0;
        for (int k = 0; k < m && warp < NW; k++) {
            const int a = s_idx[k];
            const int* row = nbr + (size_t)a * cap;
            const int u = nup[a], l = nlo[a], n14 = c14s[a + 1] - c14s[a];
            const int cnt = u + l + n14;
            int q = (gslot - 2 * base) % G;
            if (q < 0) q += G;
            for (; q < 2 * cnt; q += G) {
                const int t = q >> 1, side = q & 1;
                const bool fourteen = t >= u + l;
                const int j = fourteen ? c14d[c14s[a] + t - u - l] : (t < u ? row[t] : row[cap - 1 - (t - u)]);
                const int sj = slot(j);
                if (sj >= 0 && j < a) continue;   // a pair of moved atoms, counted at its lower atom
                double4_32a ai = pq[a], jj = pq[j];
                if (side) {
                    ai.x = s_xyz[3 * k]; ai.y = s_xyz[3 * k + 1]; ai.z = s_xyz[3 * k + 2];
                    if (sj >= 0) { jj.x = s_xyz[3 * sj]; jj.y = s_xyz[3 * sj + 1]; jj.z = s_xyz[3 * sj + 2]; }
                }
                double e, v;
                pair_energy<PREC_F64>(A, pbc, cut, fourteen, ai, f0, a, jj, f0, j, true, e, v);
                del += side ? e : -e;
                dvd += side ? v : -v;
            }
            base += cnt;
        }
        del = warp_sum(del);
        dvd = warp_sum(dvd);
        if (lane == 0 && warp < NW) { s_part[0][warp] = del; s_part[1][warp] = dvd; }
        __syncthreads();
        if (tid == 0) {
            double se = 0.0, sv = 0.0;
            for (int w = 0; w < NW; w++) { se += s_part[0][w]; sv += s_part[1][w]; }
            for (int r = 0; r < RP_CL; r++) *cluster.map_shared_rank(&s_cl[rank], r) = make_double2(se, sv);
        }
        cluster.sync();
        if (tid == 0) {
            double se = 0.0, sv = 0.0;
            for (int r = 0; r < RP_CL; r++) { se += s_cl[r].x; sv += s_cl[r].y; }
            const double de = CHGCHARMM * KCALTOIU * se + 4.0 * sv;
            // MC_metropolis::apply_criterion (MC_metropolis.cpp:175-204); exp is CUDA's (at most 1 ulp
            // from the exact value) where the host loop calls glibc's: the two runs can part only on a
            // uniform within an ulp of the threshold
            long long cur = s_cur;
            bool accepted;
            if (de <= 2.220446049250313e-16) accepted = true;
            else accepted = rp_canonical(s_words, cur) < exp(-beta * de);
            S.cursor = cur;
            const int t = s_type;
            if (accepted) {
                S.acc_tmp[t]++;
                S.etot += de;
                S.acc++;
            }
            for (int tt = 0; tt < T.nmvtyp; tt++) {
                if (T.each[tt] != 0 && (step % T.each[tt]) == 0) {
                    const double ratio = (double)S.acc_tmp[tt] / (double)T.each[tt];
                    S.dmax[tt] = ratio > T.target[tt] / 100 ? S.dmax[tt] * 1.10 : S.dmax[tt] * 0.9;
                    S.acc_tmp[tt] = 0;
                }
            }
            S.steps_done = step;
            s_acc = accepted ? 1 : 0;
        }
        __syncthreads();
        if (s_acc && rank == 0) {
            for (int k = tid; k < m; k += blockDim.x) {
                const int a = s_idx[k];
                double4_32a p = pq[a];
                p.x = s_xyz[3 * k]; p.y = s_xyz[3 * k + 1]; p.z = s_xyz[3 * k + 2];
                pq[a] = p;
                uint4 f = fx[a];
                f.x = to_fixed(p.x, pbc.rL[0]); f.y = to_fixed(p.y, pbc.rL[1]); f.z = to_fixed(p.z, pbc.rL[2]);
                fx[a] = f;
            }
            __threadfence();
        }
        cluster.sync();   // the commit before the next step's reads; every CTA is past this step's sums
    }
    if (tid == 0 && rank == 0) *st = S;
}

bool SingleEngine::replay_cluster_ok() {
    static int ok = -1;
    if (ok < 0) {
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3(RP_CL);
        cfg.blockDim = dim3(RP_NT + RP_SPEC);
        int nclusters = 0;
        ok = cudaOccupancyMaxActiveClusters(&nclusters, k_replay, &cfg) == cudaSuccess && nclusters >= 1 ? 1 : 0;
        if (!ok) cudaGetLastError();
    }
    return ok == 1;
}

int SingleEngine::metropolis_device(std::mt19937& gen, const std::vector<MoveKind>& moves, double beta, int nsteps,
                                    double* etot, int64_t* n_accepted) {
    const int nt = (int)moves.size();
    if (nt < 1 || nt > RP_MAXT) return fail(MCG_ENOTSUP, "device run: 1 to 8 move types");
    ReplayTables T{};
    ReplayState S{};
    std::vector<int> first, ranges;
    T.nmvtyp = nt;
    for (int t = 0; t < nt; t++) {
        const MoveKind& mk = moves[t];
        T.ninst[t] = mk.ninst();
        T.ibase[t] = (int)first.size();
        T.each[t] = mk.each;
        T.target[t] = mk.target;
        S.dmax[t] = mk.dmax;
        const int rb = (int)ranges.size() / 2;
        for (int k = 0; k < mk.ninst(); k++) first.push_back(rb + mk.rstart[k]);
        ranges.insert(ranges.end(), mk.ranges.begin(), mk.ranges.end());
    }
    first.push_back((int)ranges.size() / 2);
    S.etot = *etot;
    constexpr long long W = RP_WORDS;        // random words per launch
    int* d_first = nullptr;
    int* d_ranges = nullptr;
    uint32_t* d_words = nullptr;
    ReplayState* d_st = nullptr;
    int rc = MCG_OK;
    auto done = [&](int r) {
        if (d_first) cudaFree(d_first);
        if (d_ranges) cudaFree(d_ranges);
        if (d_words) cudaFree(d_words);
        if (d_st) cudaFree(d_st);
        return r;
    };
    if ((rc = dalloc(&d_first, first.size())) || (rc = dalloc(&d_ranges, std::max<size_t>(1, ranges.size()))) ||
        (rc = dalloc(&d_words, (size_t)W)) || (rc = dalloc(&d_st, 1)))
        return done(rc);
    if (cudaMemcpyAsync(d_first, first.data(), sizeof(int) * first.size(), cudaMemcpyHostToDevice, stream) != cudaSuccess ||
        (!ranges.empty() &&
         cudaMemcpyAsync(d_ranges, ranges.data(), sizeof(int) * ranges.size(), cudaMemcpyHostToDevice, stream) != cudaSuccess))
        return done(fail(MCG_ECUDA, "device run: table upload"));
    T.inst_first = d_first;
    T.ranges = d_ranges;
    T.ninst_all = (int)first.size();
    T.nranges = (int)ranges.size() / 2;
    std::vector<uint32_t> w((size_t)W);
    std::vector<uint32_t> stash;     // the generator's next words, drawn while the previous launch ran
    size_t stash_at = 0;
    long long filled = 0;
    int step = 0;
    while (step < nsteps) {
        // the words not consumed yet, then the generator's next ones (from the stash first)
        const long long keep = filled - S.cursor;
        if (keep > 0 && S.cursor > 0) std::memmove(w.data(), w.data() + S.cursor, sizeof(uint32_t) * (size_t)keep);
        filled = std::max(0LL, keep);
        while (filled < W) w[(size_t)filled++] = stash_at < stash.size() ? stash[stash_at++] : gen();
        S.cursor = 0;
        S.status = 0;
        const int s1 = std::min(nsteps, (step / 50 + 1) * 50);     // up to the next list update
        if (cudaMemcpyAsync(d_words, w.data(), sizeof(uint32_t) * (size_t)W, cudaMemcpyHostToDevice, stream) != cudaSuccess ||
            cudaMemcpyAsync(d_st, &S, sizeof S, cudaMemcpyHostToDevice, stream) != cudaSuccess)
            return done(fail(MCG_ECUDA, "device run: upload"));
        k_replay<<<RP_CL, RP_NT + RP_SPEC, 0, stream>>>(atoms(), d_pq, d_fx, pbc, cut, d_nbr, d_nup, d_nlo, cap, d_c14s, d_c14d, T,
                                              d_words, W, d_st, step, s1, beta);
        launches++;
        // while the launch runs: the next W words of the generator, in order, for the next buffer
        stash.erase(stash.begin(), stash.begin() + (long)stash_at);
        stash_at = 0;
        while ((long long)stash.size() < W) stash.push_back(gen());
        if (cudaGetLastError() != cudaSuccess ||
            cudaMemcpyAsync(&S, d_st, sizeof S, cudaMemcpyDeviceToHost, stream) != cudaSuccess ||
            cudaStreamSynchronize(stream) != cudaSuccess)
            return done(fail(MCG_ECUDA, "device run: replay kernel"));
        if (S.status == 2) return done(fail(MCG_ENOTSUP, "device run: a move of more than 64 atoms"));
        step = S.steps_done;
        if (S.status == 0 && step % 50 == 0) {
            if ((rc = update_lists())) return done(rc);
        }
    }
    // host mirror of the coordinates
    std::vector<double4_32a> pqh((size_t)n);
    if (cudaMemcpy(pqh.data(), d_pq, sizeof(double4_32a) * (size_t)n, cudaMemcpyDeviceToHost) != cudaSuccess)
        return done(fail(MCG_ECUDA, "device run: coordinates"));
    for (int a = 0; a < n; a++) { host_x[a] = pqh[a].x; host_y[a] = pqh[a].y; host_z[a] = pqh[a].z; }
    prune_dirty = true;
    pending_m = 0;
    *etot = S.etot;
    *n_accepted = S.acc;
    return done(MCG_OK);
}

int SingleEngine::commit() {
    if (pending_m <= 0) return fail(MCG_EINVAL, "no pending proposal to commit");
    // the pending proposal is still staged on the device: only delta_e writes d_stage, and each
    // delta_e call replaces the pending proposal.  Stream order puts the update before any later
    // call's work, so the host does not wait for it.
    const int* didx = (const int*)d_stage;
    const double* dxyz = (const double*)((char*)d_stage + pending_off_xyz);
    MoveInline inl;
    inl.m = 0; inl.nterms = 0;
    if (pending_inline) {
        inl.m = pending_m;
        memcpy(inl.idx, pending_idx.data(), 4 * (size_t)pending_m);
        memcpy(inl.xyz, pending_xyz.data(), 24 * (size_t)pending_m);
    }
    k_commit<0><<<(pending_m + 127) / 128, 128, 0, stream>>>(pending_m, didx, dxyz, d_pq, d_fx, pbc, inl);
    CK(cudaGetLastError());
    for (int k = 0; k < pending_m; k++) {
        int a = pending_idx[k];
        host_x[a] = pending_xyz[3 * k]; host_y[a] = pending_xyz[3 * k + 1]; host_z[a] = pending_xyz[3 * k + 2];
        if (!prune_dirty) note_moved(a);
    }
    pending_m = 0;
    launches += 1;
    return MCG_OK;
}

bool SingleEngine::pending_matches(int m, const int* atoms, const double* x, const double* y, const double* z) const {
    if (pending_m != m) return false;
    for (int k = 0; k < m; k++) {
        const int a = atoms[k];
        if (pending_idx[k] != a || pending_xyz[3 * k] != x[a] || pending_xyz[3 * k + 1] != y[a] ||
            pending_xyz[3 * k + 2] != z[a])
            return false;
    }
    return true;
}

int SingleEngine::update_lists() {
    if (hs.cut != MCG_CUT_SWITCH) return MCG_OK;
    int rc = build_list();
    launches += 5;
    return rc;
}

int SingleEngine::get_pairlist(int* counts, int* entries, int64_t cap_entries, int64_t* total) {
    if (hs.cut != MCG_CUT_SWITCH) {
        for (int i = 0; i < n; i++) counts[i] = 0;
        if (total) *total = 0;
        return MCG_OK;
    }
    std::vector<int> up(n);
    CK(cudaMemcpyAsync(up.data(), d_nup, sizeof(int) * n, cudaMemcpyDeviceToHost, stream));
    std::vector<int> rows((size_t)n * cap);
    CK(cudaMemcpyAsync(rows.data(), d_nbr, sizeof(int) * (size_t)n * cap, cudaMemcpyDeviceToHost, stream));
    CK(cudaStreamSynchronize(stream));
    int64_t t = 0;
    for (int i = 0; i < n; i++) { counts[i] = up[i]; t += up[i]; }
    if (total) *total = t;
    if (entries && cap_entries >= t) {
        int64_t p = 0;
        for (int i = 0; i < n; i++) {
            int* r = rows.data() + (size_t)i * cap;
            std::sort(r, r + up[i]);
            memcpy(entries + p, r, sizeof(int) * up[i]);
            p += up[i];
        }
    }
    return MCG_OK;
}

}  // namespace mcg
