// Allocation-free variant of the FP64 switched nonbonded energy over a half Verlet list.
//
// Some callers cannot allocate device memory at the moment they need an energy: host codes that
// hand every byte of the GPU to their own memory pool and forbid side allocations, and tight
// real-time loops that cannot afford cudaMalloc's implicit device synchronisation and driver lock.
// mcg_energy_switch_fp64_noalloc serves them: the caller passes device inputs and a device
// output, and the per-block partial sums live in a file-scope static device array of fixed size,
// so no call to this entry point allocates anything.
//
// Scratch: g_noalloc_partials holds two doubles per block; one block covers 8 atoms, so the
// array bounds the system at MCG_NOALLOC_MAX_ATOMS atoms (512 KiB, held by every GPU that loads
// the library until the process exits).  Every call overwrites the partials of all blocks it
// launches before they are read, so nothing has to start at zero.  All calls share the array:
// calls that overlap on the GPU (different streams, or different host threads on one device)
// race on it and must be serialised by the caller.
//
// The neighbour rows come from the caller, not from this library, so the kernel trusts none of
// their contents: a row count above the row capacity is clamped to it and a partner index outside
// [0, natom) is skipped, so a damaged list can give a wrong energy but never an access outside the
// caller's buffers.
#include <mutex>
#include <string>

#include <cuda_runtime.h>

#include "engine.hpp"
#include "mcg.h"
#include "pair_math.cuh"

namespace mcg {

constexpr int NOALLOC_ROWS_PER_BLOCK = 8;    // one warp per row, 256 threads
constexpr int NOALLOC_MAX_BLOCKS = MCG_NOALLOC_MAX_ATOMS / NOALLOC_ROWS_PER_BLOCK;

static __device__ __align__(256) double g_noalloc_partials[2 * NOALLOC_MAX_BLOCKS];

// Each block sums the switched pair terms of its 8 rows (a warp per row, lanes over the row's
// j > i entries) and writes (elec, vdw) unscaled to its own slot of the static scratch.
__global__ void __launch_bounds__(256) k_noalloc_energy(const double4_32a* __restrict__ pq, const double2* __restrict__ es,
                                                        const int* __restrict__ nbr, const int* __restrict__ nup, int n,
                                                        int cap, PbcDev pbc, CutDev cut, double* partials) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int i = blockIdx.x * NOALLOC_ROWS_PER_BLOCK + w;
    double sel = 0.0, svd = 0.0;
    if (i < n) {
        const double4_32a pi = pq[i];
        const double2 ai = es[i];
        const int* row = nbr + (size_t)i * cap;
        const int m = min(nup[i], cap);
        for (int k = lane; k < m; k += 32) {
            const int j = row[k];
            if ((unsigned)j >= (unsigned)n) continue;   // not an atom of this system
            const double4_32a pj = pq[j];
            const double r2 = ref64_dist2(pi.x, pi.y, pi.z, pj.x, pj.y, pj.z, pbc);
            if (r2 > cut.c2) continue;
            const double2 aj = es[j];
            double el, vd;
            ref64_pair(r2, pi.w, pj.w, ai.x, aj.x, ai.y, aj.y, true, cut, el, vd);
            sel += el;
            svd += vd;
        }
    }
    __shared__ double sa[8], sb[8];
    sel = warp_sum(sel);
    svd = warp_sum(svd);
    if (lane == 0) { sa[w] = sel; sb[w] = svd; }
    __syncthreads();
    if (threadIdx.x == 0) {
        double a = 0.0, b = 0.0;
        for (int k = 0; k < NOALLOC_ROWS_PER_BLOCK; k++) { a += sa[k]; b += sb[k]; }
        partials[2 * blockIdx.x] = a;
        partials[2 * blockIdx.x + 1] = b;
    }
}

// One block reduces the partials in a fixed order and scales them as FField_MDBAS does
// (elec = 332.0716 * 418.4 * sum, vdw = 4 * sum; FField_MDBAS.cpp:420-421).
__global__ void k_noalloc_finalize(const double* __restrict__ partials, int nblocks, double* out) {
    __shared__ double sa[256], sb[256];
    double a = 0.0, b = 0.0;
    for (int k = threadIdx.x; k < nblocks; k += blockDim.x) { a += partials[2 * k]; b += partials[2 * k + 1]; }
    sa[threadIdx.x] = a;
    sb[threadIdx.x] = b;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) { sa[threadIdx.x] += sa[threadIdx.x + o]; sb[threadIdx.x] += sb[threadIdx.x + o]; }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        out[0] = CHGCHARMM * KCALTOIU * sa[0];
        out[1] = 4.0 * sb[0];
    }
}

// Device address of the static scratch, looked up once per device with that device current and
// kept for the process.  The table is guarded by a mutex, so host threads may call concurrently.
// A cudaDeviceReset() of the device unloads the module and makes the kept address stale; callers
// that reset a device must not call this entry point on it afterwards.
static double* noalloc_scratch(int dev, int* rc) {
    static std::mutex mu;
    static double* addr[64] = {nullptr};
    if (dev < 0 || dev >= 64) { *rc = fail(MCG_ENOTSUP, "device ordinal above 63"); return nullptr; }
    std::lock_guard<std::mutex> lock(mu);
    if (!addr[dev]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_partials);
        if (e != cudaSuccess) {
            cudaGetLastError();   // this call's own error: not left pending for the caller's next call
            *rc = fail(MCG_ECUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
            return nullptr;
        }
        addr[dev] = (double*)p;
    }
    *rc = MCG_OK;
    return addr[dev];
}

}  // namespace mcg

extern "C" int mcg_energy_switch_fp64_noalloc(int natom, const double* pq, const double* es, const int* nbr,
                                              const int* nup, int cap, int pbc_type, const double box[3],
                                              double cutoff, double cuton, double* out, void* stream) {
    using namespace mcg;
    if (natom <= 0 || natom > MCG_NOALLOC_MAX_ATOMS)
        return fail(MCG_EINVAL, "natom must be in [1, " + std::to_string(MCG_NOALLOC_MAX_ATOMS) + "] for the allocation-free energy");
    if (!pq || !es || !nbr || !nup || !out || !box) return fail(MCG_EINVAL, "null argument");
    if (cap <= 0) return fail(MCG_EINVAL, "row capacity must be positive");
    if (((uintptr_t)pq & 31) || ((uintptr_t)es & 15)) return fail(MCG_EINVAL, "pq must be 32-byte and es 16-byte aligned");
    if (pbc_type < MCG_PBC_NONE || pbc_type > MCG_PBC_ORBIC) return fail(MCG_EINVAL, "bad pbc_type");
    if (!(cutoff > cuton) || !(cuton >= 0)) return fail(MCG_EINVAL, "need cutoff > cuton >= 0");
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) { cudaGetLastError(); return fail(MCG_ECUDA, "no CUDA device available"); }
    int rc;
    double* scratch = noalloc_scratch(dev, &rc);
    if (!scratch) return rc;
    PbcDev pbc;
    pbc.type = pbc_type;
    for (int k = 0; k < 3; k++) {
        double L = pbc_type == MCG_PBC_CUBIC ? box[0] : box[k];
        if (pbc_type != MCG_PBC_NONE && !(L > 0)) return fail(MCG_EINVAL, "box lengths must be positive");
        pbc.L[k] = pbc_type != MCG_PBC_NONE ? L : 0.0;
        pbc.rL[k] = pbc_type != MCG_PBC_NONE ? 1.0 / L : 0.0;
    }
    CutDev cut;
    cut.mode = 1;
    cut.c2 = cutoff * cutoff;
    cut.n2 = cuton * cuton;
    {
        double d = cut.c2 - cut.n2;
        cut.sw2 = 1. / (d * d * d);
    }
    cut.c2f = (float)cut.c2; cut.n2f = (float)cut.n2; cut.sw2f = (float)cut.sw2;
    cudaStream_t st = (cudaStream_t)stream;
    const int nblocks = (natom + NOALLOC_ROWS_PER_BLOCK - 1) / NOALLOC_ROWS_PER_BLOCK;
    // launched through cudaLaunchKernel, whose return value is this launch's own status: an error
    // left by the caller's earlier asynchronous work is neither reported here nor cleared
    const double4_32a* a_pq = (const double4_32a*)pq;
    const double2* a_es = (const double2*)es;
    int a_n = natom, a_cap = cap, a_nb = nblocks;
    void* args1[] = {(void*)&a_pq, (void*)&a_es, (void*)&nbr, (void*)&nup, (void*)&a_n, (void*)&a_cap, (void*)&pbc,
                     (void*)&cut, (void*)&scratch};
    cudaError_t e = cudaLaunchKernel((const void*)k_noalloc_energy, dim3(nblocks), dim3(256), args1, 0, st);
    if (e == cudaSuccess) {
        void* args2[] = {(void*)&scratch, (void*)&a_nb, (void*)&out};
        e = cudaLaunchKernel((const void*)k_noalloc_finalize, dim3(1), dim3(256), args2, 0, st);
    }
    if (e != cudaSuccess) {
        cudaGetLastError();   // the failed launch's error is reported here, not left for the next call
        return fail(MCG_ECUDA, std::string("launch: ") + cudaGetErrorString(e));
    }
    return MCG_OK;
}
