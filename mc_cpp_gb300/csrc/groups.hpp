// Group-pair form of the (pruned) Verlet half list, for the mixed-precision switched energy of
// periodic boxes.
//
// A group is a run of at most 4 consecutive atoms of one residue (a water molecule is one group).
// Each Verlet pair (i, j), j > i, of the rows the pair kernel reads becomes one bit (a * 4 + b,
// a = i's slot in its group, b = j's slot) of a 16-bit mask on the group pair (group(i),
// group(j)), stored in the row of group(i); group(j) >= group(i) always, since groups are runs of
// consecutive atoms.  So the set of pairs evaluated is that of the rows exactly (stale rows,
// exclusions and frozen pairs included).  The energy kernel takes a warp per group row: the
// group's atoms stay in registers, and each lane takes one entry of the row, gathers the entry's
// atoms as one contiguous run (one index per up to 4 atoms, instead of one per atom) and
// evaluates the entry's masked atom pairs.
#pragma once
#include <cstdint>
#include <vector>

#include <cuda_runtime.h>

namespace mcg {

// Geometry and cutoff constants of the group-pair energy kernel.
struct GroupGeom {
    float Ls[3], Ll[3];   // box / 2^32 as float-float (fixed-point displacement scale)
    float L2h, L2l;       // (box / 2^32)^2 as float-float (cubic boxes: r^2 in fixed-point units)
    float c2, n2, k3;     // rc^2, ron^2, rc^2 - 3 ron^2 (FP32)
    double inv_f1;        // 1 / (the FP32 switch polynomial at r^2 <= ron^2): makes inner pairs exactly 1
    float D;              // rc^2 - ron^2 (FP32)
    double inv_p1;        // 1 / (the packed kernels' polynomial u^2 (3D - 2u) at u = D, in FP32 as they form it)
    float emax;           // half the smallest box edge less rc (and 1e-3 A): a row group whose atoms lie
                          // within emax of its first atom (each component) sees every partner within rc
                          // at its minimum image relative to that first atom
    int iso;              // cubic box: r^2 summed in fixed-point units
};

class GroupPairs {
public:
    ~GroupPairs() { release(); }
    // Groups from the residue ids (host, once): runs of consecutive atoms with one residue id,
    // cut every 4 atoms.
    int setup(const std::vector<int>& resid);
    // Rebuilds the group rows from the per-atom rows (rows: n rows of stride cap, lens[i] entries
    // each, all j > i).  Returns MCG_OK, or a failure status; on MCG_ECAPACITY the path is marked
    // unavailable and the caller keeps the per-atom list kernels.
    int build(cudaStream_t st, const int* rows, const int* lens, int cap);
    // Energy kernel, variant v of kVariants: writes 2 doubles (elec, vdw, unscaled as k_finalize
    // expects) per CTA into part and returns the number of CTAs.  Needs the parameter-class table
    // (cls, ncls > 0).
    int launch_energy(cudaStream_t st, int v, const uint4* fx, const float4* cls, int ncls, const GroupGeom& G,
                      double* part);
    static constexpr int kVariants = 4;

    bool ok = false;
    int n = 0, ngroup = 0, gcap = 0;
    int gmax = 1;                // largest group (atoms)
    int64_t nentries = 0;        // group pairs in the rows
    int64_t nbits = 0;           // atom pairs their masks encode (the source rows' size)
    int64_t build_launches = 0;

private:
    void release();
    int *d_gstart = nullptr;     // first atom of each group (ngroup + 1)
    int *d_gof = nullptr;        // group of each atom
    int2* d_grow = nullptr;      // group rows: (first atom of the partner group, mask | (size - 1) << 16)
    int* d_glen = nullptr;       // entries per group row
    unsigned long long* d_misc = nullptr;   // [0] entries, [1] mask bits, [2] overflow flag
    size_t grow_cap = 0;
};

}  // namespace mcg
