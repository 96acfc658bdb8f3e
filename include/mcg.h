/*
 * mcg.h — C ABI of the GB300 nonbonded Monte Carlo energy engine (libmcgpu.so).
 *
 * This is the drop-in boundary for FHedin/mc_cpp's energy path: every entry point below replaces
 * one member of the reference's FField / List_nonBonded / MC_metropolis call graph or of its
 * existing C ABI (src/FORTRAN_interface.cpp).  Plain pointers and sizes only; no C++ or CUDA types
 * cross this boundary.  All energies are in the reference's internal units
 * (1 kcal/mol = 418.4 iu, include/Constants.hpp:29) unless a function says otherwise.
 *
 * Error convention: every function returns an int status, MCG_OK (0) or a negative MCG_E* code,
 * and never exits the process.  mcg_last_error() describes the most recent failure of the calling
 * thread.  (The reference prints to cerr and calls exit(); the C++ adapter FField_CUDA maps a
 * non-zero status back to that convention.)
 *
 * Threading: a handle is single-owner; calls on one handle must not overlap.  Each handle owns one
 * CUDA stream on the device that was current when it was created.
 */
#ifndef MCG_H
#define MCG_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MCG_ABI_VERSION 1

enum mcg_status {
    MCG_OK = 0,
    MCG_EINVAL = -1,     /* invalid argument or inconsistent system description */
    MCG_ECUDA = -2,      /* CUDA runtime error (no device, out of memory, launch failure) */
    MCG_ECAPACITY = -3,  /* a fixed-capacity device structure overflowed and could not grow */
    MCG_ETIMEOUT = -4,   /* a bounded device-side wait gave up */
    MCG_ENOTSUP = -5,    /* feature combination not supported */
    MCG_EIO = -6         /* file could not be read or parsed */
};

enum mcg_pbc { MCG_PBC_NONE = 0, MCG_PBC_CUBIC = 1, MCG_PBC_ORBIC = 2 };
enum mcg_cut { MCG_CUT_FULL = 0, MCG_CUT_SWITCH = 1 };
enum mcg_precision {
    MCG_PREC_FP64 = 0,   /* plain: every pair term in FP64, reference arithmetic */
    MCG_PREC_MIXED = 1   /* FP32 pair terms on exact displacements, FP64 accumulation */
};
enum mcg_move_type { MCG_MOVE_TRN = 1, MCG_MOVE_ROT = 2 };
enum mcg_move_mode { MCG_MODE_RESIDUE = 0, MCG_MODE_ALL = 1, MCG_MODE_ATOM = 2 };
enum mcg_acceptance {
    MCG_ACCEPT_REFERENCE = 0, /* beta in mol/kcal applied to dE in iu, as MC_metropolis.cpp:188 */
    MCG_ACCEPT_PHYSICAL = 1   /* beta applied to dE in kcal/mol */
};

enum mcg_units {
    MCG_UNITS_FILE = 0,       /* forcefield-file units, converted here as IO_MDBAS::read_ff does */
    MCG_UNITS_INTERNAL = 1    /* already converted (AtomList / Bond / Angle / Dihedral after IO_MDBAS):
                                 eps = sqrt(eps_file * 418.4), k in iu, theta0 and phi0 in radians */
};

/* One system: what the reference's Parser_XML + IO_MDBAS build (AtomList, PerConditions,
 * Ens_NVT, FField cut settings and the bonded lists).  Per-atom arrays have natom entries; topology
 * arrays hold 0-based atom indices; parameters are in forcefield-file units (kcal/mol, Angstrom,
 * degrees) and are converted exactly as IO_MDBAS::read_ff does (src/IO_MDBAS.cpp:186-467), unless
 * param_units says they are converted already.  Zero-initialise the struct: new fields default
 * to 0. */
typedef struct mcg_system_desc {
    int natom;
    const double *x, *y, *z;
    const double *q;
    const double *eps, *sig;        /* file epsilon (kcal/mol, stored as sqrt(eps*418.4)); MDBAS half-sigma */
    const double *eps14, *sig14;
    const double *mass;             /* may be NULL (all 1); used for centre-of-mass rotation pivots */
    const unsigned char *frozen;    /* may be NULL (none frozen) */
    const int *resid;               /* global residue ids, 1-based and consecutive; may be NULL */
    int pbc_type;                   /* enum mcg_pbc */
    double box[3];                  /* a, b, c (cubic uses a) */
    int cut_mode;                   /* enum mcg_cut */
    double cutoff, cuton, dcut;     /* switch: rc, ron, Verlet skin (reference defaults 12, 10, 2) */
    double temp;                    /* K */
    int precision;                  /* enum mcg_precision */
    int nbond;  const int *bond_atoms;  const int *bond_type;  const double *bond_k, *bond_r0, *bond_beta;
    int nub;    const int *ub_atoms;    const double *ub_k, *ub_r0;
    int nangle; const int *angle_atoms; const int *angle_type; const double *angle_k, *angle_theta0;
    int ndihe;  const int *dihe_atoms;  const int *dihe_type, *dihe_order; const double *dihe_k, *dihe_phi0, *dihe_mult;
    int nimpr;  const int *impr_atoms;  const int *impr_type, *impr_order; const double *impr_k, *impr_phi0, *impr_mult;
    int param_units;                /* enum mcg_units: how eps/eps14, force constants and angles are given */
} mcg_system_desc;

typedef struct mcg_system mcg_system;

int mcg_abi_version(void);
const char* mcg_last_error(void);
/* Number of CUDA devices visible to the library (0 without a GPU); never fails. */
int mcg_device_count(void);

/* --- single system: FField_CUDA's engine ------------------------------------------------------
 * mcg_create replaces `new FField_MDBAS(...)` + `new List_nonBonded(...)` + `setExcl`
 * (src/Parser.cpp:139-153,210-211): builds exclusion and 1-4 lists on the host
 * (List_nonBonded::build_exclude_list, src/List_nonBonded.cpp:143-775) and, in switch mode, the
 * Verlet list on the device (init/update_verlet_list, :777-915). */
int mcg_create(const mcg_system_desc* desc, mcg_system** out);
int mcg_destroy(mcg_system* s);

/* AtomList::setCoords for all atoms (src/FORTRAN_interface.cpp:77-82 set_coords_). */
int mcg_set_coords(mcg_system* s, const double* x, const double* y, const double* z);
int mcg_get_coords(mcg_system* s, double* x, double* y, double* z);

/* FField::getE(double ener[10]) (src/FField_MDBAS.cpp:77-106): full recompute on the device with
 * the current list; ener = [tot, pot, kin(=0), elec, vdw, bond, ang, ub, dihe, impr] in iu. */
int mcg_energy(mcg_system* s, double ener[10]);

/* FField::getE() (src/FField_MDBAS.cpp:53-75) for a caller that moves atoms in place between calls,
 * as MC_metropolis::run does around every trial move (src/MC_metropolis.cpp:94,122,130-133):
 * x, y, z are the caller's current coordinates of all atoms and *etot receives their total energy
 * (iu).  Only what changed since the engine's coordinates is sent to the device: nothing when no
 * atom moved; a commit of the last proposal when exactly its atoms sit at its coordinates (an
 * accepted move); the dE of the changed atoms (at most 1024, as mcg_delta_e) when a new move was
 * made; a full upload and recompute otherwise, and on the first call after mcg_create,
 * mcg_set_coords, mcg_commit, mcg_update_lists or a Metropolis run.  The total then carries the
 * dE sums since that recompute (mcg_delta_e's error per move, none in FP64 beyond rounding). */
int mcg_energy_host(mcg_system* s, const double* x, const double* y, const double* z, double* etot);

/* FField::askListUpdate (src/FField.cpp:222-235): rebuild the Verlet list from the current
 * coordinates with a device cell list.  No-op in full mode. */
int mcg_update_lists(mcg_system* s);

/* Energy change of moving atoms[0..n) to (nx,ny,nz), nonbonded (current list, same cutoff, switch,
 * exclusion and 1-4 rules as mcg_energy) plus the bonded terms that touch them.  Equals
 * E(after) - E(before) as the reference computes it in MC_metropolis.cpp:94-123 (two getE calls),
 * without its cancellation error.  The proposal is kept until the next mcg_delta_e / mcg_commit.
 * 1 <= n <= 1024. */
int mcg_delta_e(mcg_system* s, int n, const int* atoms, const double* nx, const double* ny,
                const double* nz, double* de);
/* Apply the last proposal's coordinates on the device (an accepted move). */
int mcg_commit(mcg_system* s);

/* Half Verlet list of the current build: for each atom i the partners j > i (List_nonBonded
 * getNeighPair/getNeighList).  counts[natom] always filled; entries (row-concatenated, each row
 * sorted ascending) filled when cap is large enough; *total = sum(counts). */
int mcg_get_pairlist(mcg_system* s, int* counts, int* entries, int64_t cap, int64_t* total);
/* Pair counts of the current build.  Switch: the Verlet-list entries, and those within the cutoff
 * at the current coordinates (FP64 minimum-image distances).  Full: both are the number of pairs
 * the full energy sums (every pair i < j outside the exclusion rows). */
int mcg_pair_count(mcg_system* s, int64_t* list_pairs, int64_t* in_cutoff);
/* Kernel launches issued by the handle so far (an addition without a reference counterpart). */
int mcg_kernel_launches(mcg_system* s, int64_t* launches);
/* Device time (ms, CUDA events on the handle's stream) of reps launches of the switched
 * nonbonded pair kernel alone over the current list (switch mode). */
int mcg_time_nonbonded(mcg_system* s, int reps, float* ms);
/* The same with the L2 cache flushed before each launch (a 256 MiB device buffer written on the
 * handle's stream between launches, outside the timed intervals): *ms is the sum of the reps
 * launches' own device times.  An addition without a reference counterpart. */
int mcg_time_nonbonded_flushed(mcg_system* s, int reps, float* ms);
/* Kernel of the mixed-precision periodic switch energy (an addition without a reference
 * counterpart: FField_MDBAS has one scalar loop).  variant -1 (the default) times every variant
 * at the first energy and keeps the fastest; 0..3 are per-atom list kernels; 4 and 5 are
 * cluster-pair kernels over the cluster form of the same Verlet list; 6 to 9 are group-pair
 * kernels over the group form of the rows the list kernels read (8 and 9: packed FP32, two
 * entries per lane) (MCG_ENOTSUP when a form could
 * not be built).  mcg_get_pair_kernel reports the variant in use (-1 before the first energy) and
 * the number of variants. */
int mcg_set_pair_kernel(mcg_system* s, int variant);
int mcg_get_pair_kernel(mcg_system* s, int* variant, int* count);
/* Cluster form of the current Verlet list (mixed periodic switch systems; zeros otherwise), built
 * on demand from the list in place: clusters of 8 atoms, cluster pairs in the list, and the
 * Verlet pairs their masks encode (equal to the half-list size when the cluster list is
 * complete).  The engine builds it only for its first energy (to time the cluster kernels) and
 * while a cluster kernel is in use. */
int mcg_cluster_stats(mcg_system* s, int64_t* clusters, int64_t* cluster_pairs, int64_t* mask_pairs);
/* Group form of the rows the per-atom list kernels read (mixed periodic switch systems with at most
 * 1,024 distinct atom parameter sets; zeros otherwise), built on demand: groups (runs of at most 4
 * consecutive atoms of one residue), group pairs in the rows, and the atom pairs their masks encode
 * (equal to the rows' size: mcg_prune_stats' entries, or the half-list size without pruning). */
int mcg_group_stats(mcg_system* s, int64_t* groups, int64_t* entries, int64_t* mask_pairs);
/* Dynamic pruning of the rows the per-atom list kernels of the mixed periodic switch energy read
 * (an addition without a reference counterpart: FField_MDBAS sums its whole Verlet list).  Before
 * a launch, each half Verlet row is pruned on the device to the partners within cutoff + buffer
 * (A) of it, once after every list build and again whenever an atom has moved more than half the
 * buffer since the last prune (set_coords and commit track this on the host).  Every list pair
 * within the cutoff stays in the pruned rows, so the energy sums the same pairs as over the whole
 * list; pairs the Verlet build left out stay out.  buffer 0 turns pruning off; the default is
 * 0.5 A.  MCG_ENOTSUP for a non-zero buffer on other systems.  mcg_prune_stats reports the
 * entries of the last pruned rows, the number of prunes so far and the last prune's device time
 * (ms, CUDA events on the handle's stream); zeros before the first prune. */
int mcg_set_prune_buffer(mcg_system* s, double buffer);
int mcg_prune_stats(mcg_system* s, int64_t* entries, int64_t* prunes, float* last_ms);
/* Effective exclusion rows as the reference stores them (first exclPair[i] entries of
 * exclList[i]) and the 1-4 pair list (getNeighList14). */
int mcg_get_exclusions(mcg_system* s, int* counts, int* entries, int64_t cap, int64_t* total);
int mcg_get_pairs14(mcg_system* s, int* pairs, int cap, int* n14);
/* Host-only (no device needed): validate a description and build its exclusion rows and 1-4
 * pairs as List_nonBonded::build_exclude_list does (src/List_nonBonded.cpp:143-775). */
int mcg_build_exclusions(const mcg_system_desc* desc, int* counts, int* entries, int64_t cap, int64_t* total,
                         int* pairs14, int cap14, int* n14);

/* --- Metropolis driver: MC_metropolis::run on this engine ------------------------------------
 * Moves are registered like List_Moves::addNewMoveType (src/List_Moves.cpp:257-457);
 * sele[natom] holds the Selection flags.  mcg_metropolis_run follows MC_metropolis::run's draw
 * order with libstdc++'s mt19937 + uniform_real_distribution (MC.cpp:110-156), applies moves on
 * the host exactly as Move.hpp does, and takes dE from mcg_delta_e.  The Verlet list is rebuilt
 * every 50 steps (MC_metropolis.cpp:151).  trace (may be NULL) receives 12 doubles per step:
 * st, imvtyp, imvatm, r0, r1, r2, rang, eold, enew, de, alpha (-1 if not drawn), accepted.
 * With follow != NULL (nsteps*2 ints: imvtyp, accepted per step), accept decisions are taken from
 * it when they disagree with this engine's and the disagreement is a tie (the draw alpha within
 * 1e-6 of exp(-beta dE), or, when no alpha was drawn, |dE| <= 1e-6 iu); ties are counted in
 * *n_ties.  Any other disagreement, or a different move type, ends the run with MCG_EINVAL.
 * A run with neither trace nor follow, FP64, switched cutoff, periodic box, no bonded terms and
 * translation moves only (at most 8 types, 64 atoms a move) runs on the device: one kernel
 * launch per 50 steps draws, moves, decides and commits from the same mt19937 words, with the
 * same draws, decisions and coordinates as the host loop. */
int mcg_add_move(mcg_system* s, int type, int mode, const int* sele, double dmax, double target, int each);
int mcg_metropolis_run(mcg_system* s, int nsteps, uint64_t seed, int acceptance_units, double* trace,
                       const int* follow, double* final_etot, int64_t* n_accepted, int64_t* n_ties);
/* The same run with MC_metropolis::run's outputs (src/MC_metropolis.cpp:156-162, MC::write_traj
 * src/MC.cpp:93-108): after every save_each-th step (save_each > 0) the coordinates go to frames
 * (natom (x, y, z) triples per frame; frame k holds step (k + 1) * save_each) and the running total
 * energy (iu) to energies[k]; both hold nsteps / save_each entries. */
int mcg_metropolis_run_saving(mcg_system* s, int nsteps, uint64_t seed, int acceptance_units, int save_each,
                              double* frames, double* energies, double* final_etot, int64_t* n_accepted);

/* --- batched independent chains ----------------------------------------------------------------
 * Hundreds of NVT chains of rigid molecules (each chain: identical residues of 1..8 atoms, all
 * intra-residue pairs excluded, residue moves TRN + ROT as in MC_metropolis) advance in one
 * persistent kernel per sweep (one sweep = nres(chain) trial moves per chain), mixed precision,
 * per-chain Philox4x32-10 streams, per-chain Verlet lists rebuilt on the device when any atom
 * has moved more than half the skin.  Coordinates stay resident on the device. */
typedef struct mcg_batch mcg_batch;

typedef struct mcg_batch_opts {
    double dmax_trn;          /* Angstrom */
    double dmax_rot;          /* degrees */
    int acceptance_units;     /* enum mcg_acceptance */
    int threads_per_chain;    /* threads of the CTA that runs a chain's moves (128, 256 or 512; 0 = 512) */
    int list_capacity;        /* 0 = automatic: maximum list entries per residue */
    uint64_t seed;            /* base seed; chain c uses (seed, c) as its Philox key */
    int ctas_per_sm;          /* persistent CTAs per SM the chains are packed onto (0 = 1) */
    int speculation;          /* moves evaluated together per chain: 0 = the widest the chain's size allows, 1 = off, 2, 4, 8, 16, 32 */
    int clusters;             /* 0 = automatic (on with 512-thread CTAs): the largest chains each run on a
                                 cluster of two CTAs (two SMs); -1 = off */
    /* dmax adjustment per move type (index 0 = TRN, 1 = ROT), as MC_metropolis::run does it
     * (src/MC_metropolis.cpp:136-146, MC::adjust_dmax src/MC.cpp:165-173): after every
     * dmax_each[t]-th move of a chain (0 = never), dmax[t] is multiplied by 1.1 when the moves of
     * type t accepted since the last adjustment, divided by dmax_each[t], exceed dmax_target[t]
     * percent, else by 0.9.  Adjusted values are capped at dmax_max[t] (0 = twice the initial
     * value when adjusted, the initial value otherwise): the sweep sizes its neighbour radii for
     * the largest move, so the cap is part of the geometry. */
    int dmax_each[2];
    double dmax_target[2];
    double dmax_max[2];
} mcg_batch_opts;

/* chains[c] describes chain c (as for mcg_create; precision, cut_mode must be switch). */
int mcg_batch_create(const mcg_system_desc* chains, int nchains, const mcg_batch_opts* opts, mcg_batch** out);
int mcg_batch_destroy(mcg_batch* b);
/* Run nsweeps sweeps (one kernel launch each, replayed from a captured CUDA graph). */
int mcg_batch_sweep(mcg_batch* b, int nsweeps);
/* Same, host-synchronous, returning per-chain totals: trials, accepted, running E (iu). */
int mcg_batch_stats(mcg_batch* b, int64_t* trials, int64_t* accepted, double* etot);
/* Current dmax of every chain: translation (Angstrom) and rotation (degrees), nchains each. */
int mcg_batch_get_dmax(mcg_batch* b, double* dmax_trn, double* dmax_rot);
/* Fresh FP64 recompute of every chain's nonbonded energy (iu) with a freshly built list. */
int mcg_batch_energy_fp64(mcg_batch* b, double* e);
int mcg_batch_get_coords(mcg_batch* b, int chain, double* x, double* y, double* z);
int mcg_batch_set_coords(mcg_batch* b, int chain, const double* x, const double* y, const double* z);
/* One trial move of a logged sweep (no counterpart in the reference, whose MC_metropolis keeps no
 * per-move record): what the sweep proposed and decided, for checking it against an FP64
 * restatement of the same chain. */
typedef struct mcg_batch_move {
    double de;                  /* the move's dE (iu) as the sweep's Metropolis test used it */
    int residue;                /* moved residue, index within its chain */
    int flags;                  /* bit 0: rotation (else translation); bit 1: accepted */
    uint32_t alpha_hi, alpha_lo;/* Philox words of the acceptance draw, alpha = ((hi << 21 ^ lo >> 11) + 1) / 2^53 */
    double xyz[8][3];           /* proposed positions (A, in [-L/2, L/2)) of the residue's atoms; first apr used */
} mcg_batch_move;
/* One sweep with per-move records, host-synchronous: moves[r0(c) + k] receives chain c's k-th trial
 * move of this sweep (its Philox counter is the chain's trial count before the sweep plus k), where
 * r0(c) is the number of residues of the chains before c; cap >= the residues of all chains.  The
 * sweep runs the same kernels as mcg_batch_sweep, launched directly instead of from the graph. */
int mcg_batch_sweep_logged(mcg_batch* b, mcg_batch_move* moves, int64_t cap);
/* Run nsweeps sweeps and return their device time in milliseconds (CUDA events on the handle's
 * stream, synchronised on both sides). */
int mcg_batch_time_sweeps(mcg_batch* b, int nsweeps, float* ms);
/* Run nsweeps sweeps, each replayed from a graph that records events around its two phases, and
 * return the device time of all of them (ms_total), of the list rebuilds (k_batch_bin +
 * k_batch_lists, ms_lists) and of the sweep kernel alone (ms_sweep), summed over the sweeps.  The
 * host waits for each sweep before it reads that sweep's phase times. */
int mcg_batch_time_phases(mcg_batch* b, int nsweeps, float* ms_total, float* ms_lists, float* ms_sweep);

/* Launch shape of the sweep kernel chosen by the autotuner. */
typedef struct mcg_batch_tuning {
    int threads_per_chain;    /* 128, 256 or 512 */
    int ctas_per_sm;          /* persistent CTAs per SM (1, 2, 4 or 8) */
    int speculation;          /* cap on moves evaluated together per chain (0 = the widest the chain's size allows) */
    float ms_per_sweep;       /* device time of one sweep at that shape (0 if not measured) */
    int from_cache;           /* 1 when taken from the cache without trial sweeps */
    int clusters;             /* 1: the largest chains run on two-CTA clusters */
} mcg_batch_tuning;
/* Autotuner: times trial_sweeps sweeps (1..64) of every candidate launch shape (threads per chain
 * x CTAs per SM x speculation cap x two-CTA clusters for the largest chains) on this batch, times
 * the six fastest again in three interleaved rounds of one sweep each (the chains drift while
 * shapes are timed) and keeps the fastest.  The trial sweeps are
 * ordinary Metropolis sweeps: they advance the chains and count in their statistics.  With
 * use_cache != 0 a shape already tuned for the same workload signature (chain sizes and boxes,
 * cutoffs, move sizes, device name) in this process, or in the file named by the environment
 * variable MCG_TUNE_CACHE, is applied without trial sweeps; new results are appended there. */
int mcg_batch_autotune(mcg_batch* b, int trial_sweeps, int use_cache, mcg_batch_tuning* out);
/* Current launch shape (ms_per_sweep = 0). */
int mcg_batch_get_tuning(mcg_batch* b, mcg_batch_tuning* out);
/* Host-buffer run: when xyz_in != NULL, copy all chains' coordinates in (3*natoms doubles: x for
 * every atom of every chain, then y, then z); a chain whose coordinates differ from the device's
 * takes them, has its lists rebuilt when an atom moved beyond the rebuild threshold and its running
 * energy recomputed, while a chain given back exactly the coordinates of the last export is left
 * as it is (the FP64 view of a 64-bit fixed-point coordinate converts back to a different one, so
 * this keeps the chain's state exact); run nsweeps sweeps; when xyz_out != NULL copy the
 * coordinates back; fill accepted and etot (nchains entries each, may be NULL).  Page-locked
 * buffers (cudaHostAlloc, cudaHostRegister) are read and written by the device directly; other
 * host buffers go through a device staging copy.  Host-synchronous. */
int mcg_batch_run_host(mcg_batch* b, const double* xyz_in, int nsweeps, double* xyz_out, int64_t* accepted,
                       double* etot);
/* Mixed-precision recompute of every chain's energy over its neighbour lists (iu). */
int mcg_batch_energy_mixed(mcg_batch* b, double* e);
/* Pair interactions evaluated so far by each chain (pairs inside the cutoff before or after a move). */
int mcg_batch_pairs(mcg_batch* b, int64_t* pairs);
/* The residue neighbour lists of one chain as they are now: counts[nres] always; entries (the
 * rows concatenated, residue indices within the chain) when cap >= *total. */
int mcg_batch_get_lists(mcg_batch* b, int chain, int* counts, int* entries, int64_t cap, int64_t* total);
/* Rebuild every chain's neighbour lists now (the batched counterpart of FField::askListUpdate,
 * FField.cpp:222-235).  Sweeps rebuild lists by themselves when atoms have moved enough. */
int mcg_batch_update_lists(mcg_batch* b);
/* Exact checkpoint of a batch (no counterpart in the reference: MC::write_traj, src/MC.cpp:93-108,
 * saves frames and energies, not the random-number state).  mcg_batch_save writes every chain's
 * 64-bit fixed-point coordinates, the positions its lists were built from, its Philox counter,
 * running energy, counters, dmax state, and the launch shape, to a file (written whole, then
 * renamed into place).  mcg_batch_load restores them into a batch created from the same chain
 * descriptions and options (MCG_EINVAL otherwise; MCG_EIO for an unreadable, truncated or damaged
 * file), re-applying the saved launch shape: sweeping after a load gives bitwise the chains a run
 * without the save would have given. */
int mcg_batch_save(mcg_batch* b, const char* path);
int mcg_batch_load(mcg_batch* b, const char* path);
/* Total number of atoms over all chains, and a chain's atom count. */
int64_t mcg_batch_natoms(mcg_batch* b);
int mcg_batch_chain_natoms(mcg_batch* b, int chain);
/* Counters of the last sweeps: list rebuilds done, kernel launches issued by this handle. */
int mcg_batch_counters(mcg_batch* b, int64_t* list_rebuilds, int64_t* kernel_launches);

/* --- MDBAS input files ---------------------------------------------------------------------
 * IO_MDBAS::read_coord + read_ff (src/IO_MDBAS.cpp:77-505) on the host: a .cor coordinate file
 * and an MDBAS forcefield file read into library-owned arrays, in file units. */
typedef struct mcg_mdbas mcg_mdbas;
int mcg_mdbas_read(const char* cor_path, const char* ff_path, mcg_mdbas** out);
int mcg_mdbas_natom(const mcg_mdbas* m);
/* Point desc's atom and topology fields (natom .. impr_mult, param_units = MCG_UNITS_FILE) at m's
 * arrays, valid until mcg_mdbas_free; the run settings (pbc, box, cut, temp, precision) are left
 * as they are. */
int mcg_mdbas_fill(const mcg_mdbas* m, mcg_system_desc* desc);
int mcg_mdbas_free(mcg_mdbas* m);

/* FP32 FMA throughput of the current device in TFLOP/s, measured by an FFMA-chain kernel
 * (the denominator of the pair kernels' roofline). */
int mcg_probe_fp32_tflops(double* tflops);

/* --- allocation-free energy ------------------------------------------------------------------
 * No counterpart in the reference.  For callers that cannot allocate device memory when they need
 * an energy (a host code whose memory pool owns the whole GPU and forbids side allocations, or a
 * real-time loop that cannot afford cudaMalloc's implicit synchronisation): the FP64 switched
 * nonbonded energy over a half Verlet list, with its per-block partial sums in a fixed-size static
 * device array instead of allocated scratch.  All pointers are device pointers supplied by the
 * caller: pq[4*natom] = (x, y, z, q) per atom (32-byte aligned), es[2*natom] = (sqrt(eps*418.4),
 * MDBAS half-sigma) as the reference's AtomList stores them (16-byte aligned), nbr[natom*cap] rows
 * of partners j > i with nup[natom] entries each; out[2] receives (elec, vdw) in iu.  Launched on
 * `stream` (a cudaStream_t, NULL for the default stream), asynchronous.  natom is limited to
 * MCG_NOALLOC_MAX_ATOMS (the static scratch is 512 KiB on every GPU that loads the library).  The
 * rows are not trusted: counts above cap are clamped to cap and partners outside [0, natom) are
 * skipped.  The first call on a device looks up the scratch address (cudaGetSymbolAddress) with
 * that device current and keeps it for the process (stale after a cudaDeviceReset of that device).
 * Calls share the scratch: calls that overlap on the GPU race and must be serialised. */
#define MCG_NOALLOC_MAX_ATOMS 262144
int mcg_energy_switch_fp64_noalloc(int natom, const double* pq, const double* es, const int* nbr, const int* nup,
                                   int cap, int pbc_type, const double box[3], double cutoff, double cuton,
                                   double* out, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* MCG_H */
