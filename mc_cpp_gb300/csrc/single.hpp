// Single-system engine (host object owning the device state of one FField_CUDA).
#pragma once
#include <cstdint>
#include <random>
#include <vector>

#include <cuda_runtime.h>

#include "cluster.hpp"
#include "groups.hpp"
#include "dev_types.hpp"
#include "engine.hpp"

namespace mcg {

struct AtomsDev;
struct BondedDev;

class SingleEngine {
public:
    ~SingleEngine();
    int init(const HostSystem& hs);
    int energy(double ener[10]);
    int update_lists();
    int set_coords(const double* x, const double* y, const double* z);
    int get_coords(double* x, double* y, double* z);
    int delta_e(int m, const int* atoms, const double* nx, const double* ny, const double* nz, double* de);
    int commit();
    // MC_metropolis::run steps on the device (translation moves of atom sets without bonded terms,
    // periodic switched FP64 systems, no per-step output): random words from gen, as the host loop
    // draws them; etot in and out (iu), accepted moves out.
    int metropolis_device(std::mt19937& gen, const std::vector<MoveKind>& moves, double beta, int nsteps, double* etot,
                          int64_t* n_accepted);
    bool has_bonded_terms() const { return !term_data.empty(); }
    // limits of metropolis_device: move types, and atoms in one move instance
    static constexpr int kReplayMaxTypes = 8, kReplayMaxAtoms = 64;
    // every instance of every move within kReplayMaxAtoms atoms (and at most kReplayMaxTypes types)
    static bool replay_fits(const std::vector<MoveKind>& moves);
    // the device run's cluster can be resident on this device (checked once per process)
    static bool replay_cluster_ok();
    // true when the pending proposal moves exactly atoms[0..m) (ascending) to x/y/z[atoms[k]]
    bool pending_matches(int m, const int* atoms, const double* x, const double* y, const double* z) const;
    int get_pairlist(int* counts, int* entries, int64_t cap, int64_t* total);
    int time_nonbonded(int reps, float* ms);
    int time_nonbonded_flushed(int reps, float* ms);
    // Pair-kernel variant of the mixed periodic switch energy: -1 = chosen by timing at the first
    // use; 0..3 per-atom list kernels; 4.. cluster-pair kernels (when the cluster list exists).
    int set_pair_kernel(int v);
    int pair_kernel() const { return pair_variant; }
    static int pair_kernel_count();
    int cluster_stats(int64_t* clusters, int64_t* cluster_pairs, int64_t* mask_pairs);
    int group_stats(int64_t* groups, int64_t* entries, int64_t* mask_pairs);
    // Dynamic pruning of the rows the mixed periodic switch energy reads: buffer (A) beyond rc,
    // 0 = the pair kernel reads the Verlet rows themselves.
    int set_prune_buffer(double buffer);
    int prune_stats(int64_t* entries, int64_t* prunes, float* last_ms);
    ClusterPairs clp;
    GroupPairs grp;

    HostSystem hs;
    int n = 0;
    // host mirror of the coordinates (the device copy is the master once moves are committed)
    std::vector<double> host_x, host_y, host_z;
    int64_t launches = 0;
    int last_max_row = 0;
    int cap = 0;

private:
    int build_list();
    void release();
    AtomsDev atoms() const;
    int launch_nonbonded(double* nbp);     // returns the CTAs launched (partial sums written)
    int launch_pair_variant(int v, double* nbp);
    void tune_pair_kernel();
    int pair_variant = -1;        // mixed pair-kernel variant, chosen by timing at the first use
    BondedDev bonded() const;
    ClusterGeom cluster_geom() const;
    int ensure_part(size_t count);
    bool uses_pair_variants() const;
    int ensure_clusters();
    int prepare_pair_kernel();
    bool clp_dirty = false;       // the Verlet list changed since the cluster form was built
    int ensure_groups();
    GroupGeom group_geom() const;
    bool grp_setup = false;       // groups defined (mixed periodic switch systems with a class table)
    bool grp_dirty = false;       // the rows the pair kernel reads changed since the group rows were built
    int ensure_pruned();
    void note_moved(int atom);
    double prune_buf = 0.5;       // prune radius rc + prune_buf
    bool prune_dirty = true;      // rows to be pruned again before the next pair-kernel launch
    double prune_lim2 = 0.0;      // squared displacement since the prune that forces a new one
    int prn_cap = 0;
    int64_t prunes = 0;
    std::vector<double> prune_x, prune_y, prune_z;   // positions at the last prune
    int *d_prn = nullptr, *d_pnup = nullptr;         // pruned rows (stride cap) and their lengths
    unsigned long long* d_pkept = nullptr;
    cudaEvent_t ev_prune[2] = {nullptr, nullptr};

    cudaStream_t stream = nullptr;
    PbcDev pbc{};
    CutDev cut{};
    int n14 = 0, ntile = 0;
    double4_32a* d_pq = nullptr;
    double2 *d_es = nullptr, *d_es14 = nullptr;
    uint4* d_fx = nullptr;
    float2 *d_esf = nullptr, *d_esf14 = nullptr, *d_qf = nullptr;
    float4* d_prmf = nullptr;     // (q as float-float, eps, sig) per atom for the mixed pair kernel
    int* d_cls_of = nullptr;      // parameter class of each atom (also in the mirror's w)
    float4* d_cls = nullptr;      // the classes' (q hi, q lo, eps, sig); ncls = 0: per-atom gathers
    int ncls = 0;
    uint8_t* d_frozen = nullptr;
    int *d_xs = nullptr, *d_xd = nullptr, *d_fxs = nullptr, *d_fxd = nullptr;
    int2* d_p14 = nullptr;
    int *d_c14s = nullptr, *d_c14d = nullptr;
    BondT *d_bonds = nullptr, *d_ubs = nullptr;
    AngleT* d_angles = nullptr;
    TorsT *d_dihes = nullptr, *d_imprs = nullptr;
    int *d_nbr = nullptr, *d_nup = nullptr, *d_nlo = nullptr;
    int *d_cell_of = nullptr, *d_cell_count = nullptr, *d_cell_start = nullptr, *d_cell_fill = nullptr, *d_cell_atoms = nullptr;
    int ncell_cap = 0;
    double* d_part = nullptr;
    size_t part_cap = 0;
    unsigned* d_ticket = nullptr;
    double* h_map = nullptr;   // mapped pinned results (d_map is its device address)
    double* d_map = nullptr;
    int* d_maxrow = nullptr;
    void* h_stage = nullptr;
    void* d_stage = nullptr;
    size_t stage_bytes = 0;
    std::vector<int> term_start, term_data;
    std::vector<unsigned> term_seen;
    unsigned stamp = 0;
    int pending_m = 0;
    bool pending_inline = false;
    size_t pending_off_xyz = 0;
    std::vector<int> pending_idx;
    std::vector<double> pending_xyz;
};

}  // namespace mcg
