// Cluster-pair form of the Verlet list for the mixed-precision switched energy of periodic boxes.
//
// Atoms are grouped into clusters of 8 (columns of the box in x-y, sorted along z, cut every 8
// atoms; the last cluster of a column is padded with empty slots).  Each Verlet pair (i, j) of
// the half list becomes one bit of a 64-bit mask on the cluster pair (cluster(i), cluster(j)),
// owned by one of the two clusters, so the set of pairs evaluated is the Verlet list exactly
// (stale rows, exclusions, frozen pairs and all).  The energy kernel then evaluates 8 x 8 slot
// pairs of a cluster pair per warp (two passes of 32) from cluster-relative FP32 offsets:
// no per-pair gather of an index or a position, and no per-pair fixed-point conversion.
#pragma once
#include <cstdint>

#include <cuda_runtime.h>

#include "dev_types.hpp"

namespace mcg {

// Geometry and cutoff constants of the cluster energy kernel.
struct ClusterGeom {
    float Ls[3], Ll[3];   // box / 2^32 as float-float (fixed-point displacement scale)
    float Lf[3], iLf[3];  // box and its inverse (float), for the minimum image of wide cluster pairs
    float lim[3];         // a cluster pair whose extent along k reaches lim[k] = L[k] - rc takes the image test
    float c2, n2, k3;     // rc^2, ron^2, rc^2 - 3 ron^2 (FP32)
    float prune2;         // (rc + margin)^2: cluster pairs whose boxes are farther apart are skipped
    double inv_f1;        // 1 / (the FP32 switch polynomial at r^2 <= ron^2): makes inner pairs exactly 1
};

class ClusterPairs {
public:
    ~ClusterPairs() { release(); }
    // Rebuilds clusters and the cluster-pair list from the fixed-point coordinates and the Verlet
    // rows (nbr: n rows of `cap`, j > i from the front (nup), j < i from the back (nlo)).  Returns
    // MCG_OK, or a failure status (the path is then marked unavailable and the caller keeps the
    // per-atom list kernel).
    int build(cudaStream_t st, const uint4* fx, int n, const double L[3], const int* nbr, const int* nup,
              const int* nlo, int cap);
    // Launches the per-call pack kernel and the energy kernel (variant v of kVariants); writes
    // 2 doubles (elec, vdw, unscaled as k_finalize expects) per cluster into part, returns the
    // number of partial pairs written.
    int launch_energy(cudaStream_t st, int v, const uint4* fx, const float4* prmf, const ClusterGeom& G, double* part);
    static constexpr int kVariants = 2;

    bool ok = false;
    int ncl = 0;               // clusters
    int64_t npairs = 0;        // cluster pairs in the list
    int64_t nbits = 0;         // Verlet pairs encoded in the masks (must equal the half-list size)
    int64_t build_launches = 0;

private:
    void release();
    int ncx = 0, ncy = 0, ncol = 0, ncol_cap = 0, n_cap = 0, ncl_cap = 0, capP = 0;
    size_t cpl_cap = 0;
    int *d_col_of = nullptr, *d_col_count = nullptr, *d_col_start = nullptr, *d_ccl_start = nullptr,
        *d_col_fill = nullptr, *d_col_atoms = nullptr;
    int *d_cl_atom = nullptr, *d_cl_of = nullptr;
    uint4* d_cref = nullptr;
    float4 *d_cctr = nullptr, *d_chalf = nullptr;
    float4* d_sdat = nullptr;               // per slot: (offset, q hi), (q lo, eps, sig, 0)
    float4* d_hbox = nullptr;               // per half cluster: (centre, half extent)
    int* d_cp_count = nullptr;
    int4* d_cpl = nullptr;
    unsigned long long* d_misc = nullptr;   // [0] max column, [1] max list row, [2] mask bits, [3] pairs
    int* d_work = nullptr;                  // work counter of the energy kernel
};

}  // namespace mcg
