// C ABI (include/mcg.h) over the single-system engine, plus the host Metropolis driver that
// replays MC_metropolis::run (src/MC_metropolis.cpp:45-204) on the device energy.
//
// Built with -ffp-contract=off: the moves below are applied in FP64 on the host with the same
// operation order as Move.hpp, so the coordinates the device sees are the reference's.
#include <cfloat>
#include <cmath>
#include <algorithm>
#include <cstring>
#include <limits>
#include <memory>
#include <new>
#include <random>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "engine.hpp"
#include "mcg.h"
#include "single.hpp"

namespace mcg {
const char* last_error_cstr();
}

// What mcg_energy_host knows about the engine's current coordinates (its host mirror host_x/y/z):
// their total energy with the current list, and the delta_e proposal it made last, if any.  Every
// other entry point that changes coordinates, lists or the pending proposal updates or drops it.
struct IncrementalEnergy {
    bool valid = false;     // e_base is the total energy of host_x/y/z over the current list
    double e_base = 0.0;
    bool prop = false;      // the engine's pending proposal is the one mcg_energy_host made
    double e_prop = 0.0;    // the total energy with that proposal applied
    std::vector<int> diff;  // scratch: atoms whose caller coordinates differ from the mirror
    std::vector<double> nx, ny, nz;
};

struct mcg_system {
    mcg::SingleEngine eng;
    std::vector<mcg::MoveKind> moves;
    IncrementalEnergy inc;
};

using namespace mcg;

extern "C" {

int mcg_abi_version(void) { return MCG_ABI_VERSION; }
const char* mcg_last_error(void) { return last_error_cstr(); }

int mcg_device_count(void) {
    int c = 0;
    if (cudaGetDeviceCount(&c) != cudaSuccess) { cudaGetLastError(); return 0; }
    return c;
}

int mcg_create(const mcg_system_desc* desc, mcg_system** out) {
    if (!out) return fail(MCG_EINVAL, "null output handle");
    *out = nullptr;
    // the description is validated on the host first: an invalid one is MCG_EINVAL with or
    // without a device
    HostSystem hs;
    int rc = build_host_system(desc, hs);
    if (rc) return rc;
    if (mcg_device_count() <= 0) return fail(MCG_ECUDA, "no CUDA device available");
    std::unique_ptr<mcg_system> s(new (std::nothrow) mcg_system);
    if (!s) return fail(MCG_ECUDA, "host allocation failed");
    rc = s->eng.init(hs);
    if (rc) return rc;
    *out = s.release();
    return MCG_OK;
}

int mcg_destroy(mcg_system* s) {
    delete s;
    return MCG_OK;
}

int mcg_set_coords(mcg_system* s, const double* x, const double* y, const double* z) {
    if (!s || !x || !y || !z) return fail(MCG_EINVAL, "null argument");
    s->inc.valid = s->inc.prop = false;
    return s->eng.set_coords(x, y, z);
}

int mcg_get_coords(mcg_system* s, double* x, double* y, double* z) {
    if (!s || !x || !y || !z) return fail(MCG_EINVAL, "null argument");
    return s->eng.get_coords(x, y, z);
}

int mcg_energy(mcg_system* s, double ener[10]) {
    if (!s || !ener) return fail(MCG_EINVAL, "null argument");
    int rc = s->eng.energy(ener);
    s->inc.valid = rc == MCG_OK;
    s->inc.e_base = ener[0];
    s->inc.prop = false;
    return rc;
}

// FField::getE() for a caller that moves atoms in place between calls.  MC_metropolis::run calls
// getE() before and after every trial move (MC_metropolis.cpp:94,122) and restores the moved atoms
// of a rejected move (:130-133), so between two calls only the atoms of one move differ.  The
// caller's coordinates are compared with the engine's mirror of the device coordinates:
//   none differ                           -> the known energy, no device work;
//   exactly the last proposal's atoms, at
//   the proposal's coordinates            -> the proposal is committed (an accepted move);
//   at most 1024 atoms                    -> their dE over the current list (mcg_delta_e) is added
//                                            and kept as the new proposal;
//   more, or no known energy              -> all coordinates are uploaded and the energy recomputed.
// A list update, mcg_set_coords, mcg_commit or a Metropolis run makes the next call recompute.
int mcg_energy_host(mcg_system* s, const double* x, const double* y, const double* z, double* etot) {
    if (!s || !x || !y || !z || !etot) return fail(MCG_EINVAL, "null argument");
    SingleEngine& E = s->eng;
    IncrementalEnergy& I = s->inc;
    const int n = E.n;
    int rc;
    if (I.valid) {
        I.diff.clear();
        for (int i = 0; i < n; i++)
            if (!(x[i] == E.host_x[i] && y[i] == E.host_y[i] && z[i] == E.host_z[i])) {
                I.diff.push_back(i);
                if ((int)I.diff.size() > 1024) break;
            }
        const int m = (int)I.diff.size();
        if (m == 0) {
            *etot = I.e_base;
            return MCG_OK;
        }
        if (I.prop && E.pending_matches(m, I.diff.data(), x, y, z)) {
            if ((rc = E.commit())) { I.valid = I.prop = false; return rc; }
            I.e_base = I.e_prop;
            I.prop = false;
            *etot = I.e_base;
            return MCG_OK;
        }
        if (m <= 1024) {
            I.nx.resize(m); I.ny.resize(m); I.nz.resize(m);
            for (int k = 0; k < m; k++) { const int a = I.diff[k]; I.nx[k] = x[a]; I.ny[k] = y[a]; I.nz[k] = z[a]; }
            double de = 0.0;
            I.prop = false;
            if ((rc = E.delta_e(m, I.diff.data(), I.nx.data(), I.ny.data(), I.nz.data(), &de))) return rc;
            I.prop = true;
            I.e_prop = I.e_base + de;
            *etot = I.e_prop;
            return MCG_OK;
        }
    }
    I.valid = I.prop = false;
    if ((rc = E.set_coords(x, y, z))) return rc;
    double ener[10];
    if ((rc = E.energy(ener))) return rc;
    I.valid = true;
    I.e_base = ener[0];
    *etot = I.e_base;
    return MCG_OK;
}

int mcg_update_lists(mcg_system* s) {
    if (!s) return fail(MCG_EINVAL, "null handle");
    s->inc.valid = s->inc.prop = false;
    return s->eng.update_lists();
}

int mcg_delta_e(mcg_system* s, int n, const int* atoms, const double* nx, const double* ny, const double* nz,
                double* de) {
    if (!s || !atoms || !nx || !ny || !nz || !de) return fail(MCG_EINVAL, "null argument");
    s->inc.prop = false;
    return s->eng.delta_e(n, atoms, nx, ny, nz, de);
}

int mcg_commit(mcg_system* s) {
    if (!s) return fail(MCG_EINVAL, "null handle");
    s->inc.valid = s->inc.prop = false;
    return s->eng.commit();
}

int mcg_get_pairlist(mcg_system* s, int* counts, int* entries, int64_t cap, int64_t* total) {
    if (!s || !counts) return fail(MCG_EINVAL, "null argument");
    return s->eng.get_pairlist(counts, entries, cap, total);
}

int mcg_kernel_launches(mcg_system* s, int64_t* launches) {
    if (!s || !launches) return fail(MCG_EINVAL, "null argument");
    *launches = s->eng.launches;
    return MCG_OK;
}

int mcg_pair_count(mcg_system* s, int64_t* list_pairs, int64_t* in_cutoff) {
    if (!s || !list_pairs || !in_cutoff) return fail(MCG_EINVAL, "null argument");
    const HostSystem& h = s->eng.hs;
    const int n = h.n;
    std::vector<double> x(n), y(n), z(n);
    int r = s->eng.get_coords(x.data(), y.data(), z.data());
    if (r) return r;
    const double c2 = h.rc * h.rc;
    auto mic = [&](double d, int k) {
        // PerConditions::applyPBC: d -= L * rint(d / L), rint rounding half away from zero
        if (h.pbc == MCG_PBC_NONE) return d;
        const double t = d * h.rL[k];
        return d - h.L[k] * (double)(int64_t)(t + (t >= 0 ? 0.5 : -0.5));
    };
    auto within = [&](int i, int j) {
        const double dx = mic(x[j] - x[i], 0), dy = mic(y[j] - y[i], 1), dz = mic(z[j] - z[i], 2);
        return dx * dx + dy * dy + dz * dz <= c2;
    };
    int64_t tot = 0, inc = 0;
    if (h.cut == MCG_CUT_SWITCH) {
        std::vector<int> counts(n);
        int64_t total = 0;
        if ((r = s->eng.get_pairlist(counts.data(), nullptr, 0, &total))) return r;
        std::vector<int> ent((size_t)std::max<int64_t>(1, total));
        if ((r = s->eng.get_pairlist(counts.data(), ent.data(), total, &total))) return r;
        int64_t o = 0;
        for (int i = 0; i < n; i++)
            for (int k = 0; k < counts[i]; k++, o++) inc += within(i, ent[o]) ? 1 : 0;
        tot = total;
    } else {
        // every non-excluded pair (the full energy has no cutoff)
        tot = (int64_t)n * (n - 1) / 2 - (int64_t)h.fexclData.size();
        inc = tot;
    }
    *list_pairs = tot;
    *in_cutoff = inc;
    return MCG_OK;
}

int mcg_time_nonbonded(mcg_system* s, int reps, float* ms) {
    if (!s || !ms || reps < 1) return fail(MCG_EINVAL, "bad arguments");
    return s->eng.time_nonbonded(reps, ms);
}

int mcg_time_nonbonded_flushed(mcg_system* s, int reps, float* ms) {
    if (!s || !ms || reps < 1) return fail(MCG_EINVAL, "bad arguments");
    return s->eng.time_nonbonded_flushed(reps, ms);
}

int mcg_set_pair_kernel(mcg_system* s, int variant) {
    if (!s) return fail(MCG_EINVAL, "null argument");
    return s->eng.set_pair_kernel(variant);
}

int mcg_get_pair_kernel(mcg_system* s, int* variant, int* count) {
    if (!s || !variant || !count) return fail(MCG_EINVAL, "null argument");
    *variant = s->eng.pair_kernel();
    *count = SingleEngine::pair_kernel_count();
    return MCG_OK;
}

int mcg_cluster_stats(mcg_system* s, int64_t* clusters, int64_t* cluster_pairs, int64_t* mask_pairs) {
    if (!s || !clusters || !cluster_pairs || !mask_pairs) return fail(MCG_EINVAL, "null argument");
    return s->eng.cluster_stats(clusters, cluster_pairs, mask_pairs);
}

int mcg_group_stats(mcg_system* s, int64_t* groups, int64_t* entries, int64_t* mask_pairs) {
    if (!s || !groups || !entries || !mask_pairs) return fail(MCG_EINVAL, "null argument");
    return s->eng.group_stats(groups, entries, mask_pairs);
}

int mcg_set_prune_buffer(mcg_system* s, double buffer) {
    if (!s) return fail(MCG_EINVAL, "null argument");
    return s->eng.set_prune_buffer(buffer);
}

int mcg_prune_stats(mcg_system* s, int64_t* entries, int64_t* prunes, float* last_ms) {
    if (!s || !entries || !prunes || !last_ms) return fail(MCG_EINVAL, "null argument");
    return s->eng.prune_stats(entries, prunes, last_ms);
}

int mcg_get_exclusions(mcg_system* s, int* counts, int* entries, int64_t cap, int64_t* total) {
    if (!s || !counts) return fail(MCG_EINVAL, "null argument");
    const HostSystem& h = s->eng.hs;
    for (int i = 0; i < h.n; i++) counts[i] = h.exclCount[i];
    if (total) *total = (int64_t)h.exclData.size();
    if (entries && cap >= (int64_t)h.exclData.size())
        std::memcpy(entries, h.exclData.data(), sizeof(int) * h.exclData.size());
    return MCG_OK;
}

int mcg_get_pairs14(mcg_system* s, int* pairs, int cap, int* n14) {
    if (!s) return fail(MCG_EINVAL, "null handle");
    const HostSystem& h = s->eng.hs;
    int n = (int)h.pairs14.size() / 2;
    if (n14) *n14 = n;
    if (pairs && cap >= 2 * n) std::memcpy(pairs, h.pairs14.data(), sizeof(int) * 2 * n);
    return MCG_OK;
}

int mcg_build_exclusions(const mcg_system_desc* desc, int* counts, int* entries, int64_t cap, int64_t* total,
                         int* pairs14, int cap14, int* n14) {
    if (!counts) return fail(MCG_EINVAL, "null counts");
    HostSystem h;
    int rc = build_host_system(desc, h);
    if (rc) return rc;
    for (int i = 0; i < h.n; i++) counts[i] = h.exclCount[i];
    if (total) *total = (int64_t)h.exclData.size();
    if (entries && cap >= (int64_t)h.exclData.size())
        std::memcpy(entries, h.exclData.data(), sizeof(int) * h.exclData.size());
    int np = (int)h.pairs14.size() / 2;
    if (n14) *n14 = np;
    if (pairs14 && cap14 >= 2 * np) std::memcpy(pairs14, h.pairs14.data(), sizeof(int) * 2 * np);
    return MCG_OK;
}

int mcg_add_move(mcg_system* s, int type, int mode, const int* sele, double dmax, double target, int each) {
    if (!s) return fail(MCG_EINVAL, "null handle");
    MoveKind mk;
    int rc = build_move_kind(s->eng.hs, type, mode, sele, dmax, target, each, mk);
    if (rc) return rc;
    s->moves.push_back(std::move(mk));
    return (int)s->moves.size() - 1;
}

// MC_metropolis::run with the device ΔE.  Draw order (MC.cpp:110-156, MC_metropolis.cpp:80-165):
// move type, instance, [TRN: sphere (3 draws per try), scale | ROT: sphere, angle], then alpha
// only when dE > DBL_EPSILON.  Moves follow Move.hpp: translate then re-wrap each atom; rotate
// the raw coordinates about the pivot atom (or the centre of mass) by a Rodrigues matrix
// built from the normalised axis and an angle in degrees, then re-wrap each atom.
}  // extern "C"

// MC_metropolis::run (MC_metropolis.cpp:62-165) on this engine; with save_each > 0 the coordinates
// and the running total after every save_each-th step go to frames / energies (MC.cpp:93-108).
static int metropolis_impl(mcg_system* s, int nsteps, uint64_t seed, int acceptance_units, double* trace,
                           const int* follow, double* final_etot, int64_t* n_accepted, int64_t* n_ties,
                           int save_each, double* frames, double* energies) {
    if (!s) return fail(MCG_EINVAL, "null handle");
    if (s->moves.empty()) return fail(MCG_EINVAL, "no move types registered");  // MC.cpp:185-189
    if (nsteps < 0) return fail(MCG_EINVAL, "nsteps must be >= 0");
    s->inc.valid = s->inc.prop = false;
    SingleEngine& E = s->eng;
    const HostSystem& h = E.hs;
    const int nmvtyp = (int)s->moves.size();
    std::mt19937 gen;
    gen.seed(seed);
    std::uniform_real_distribution<double> dAlpha(0.0, 1.0), dMove(-1.0, 1.0);
    std::vector<double> dmax(nmvtyp);
    std::vector<int> accTmp(nmvtyp, 0);
    for (int t = 0; t < nmvtyp; t++) dmax[t] = s->moves[t].dmax;
    double beta = 1.0 / ((RBOLTZUI / KCALTOIU) * h.temp);
    if (acceptance_units == MCG_ACCEPT_PHYSICAL) beta /= KCALTOIU;
    double ener[10];
    int rc = E.energy(ener);
    if (rc) return rc;
    double etot = ener[0];
    int64_t acc = 0, ties = 0;
    // Without per-step output, translation moves of atom sets that carry no bonded term in a
    // periodic switched FP64 system run on the device, a launch per list-update period, on the same
    // random words (SingleEngine::metropolis_device), when its limits hold (at most 8 move types, 64
    // atoms a move, and a cluster of its 8 CTAs resident on the device, checked before the first
    // step); every other run takes the host loop below.
    bool all_trn = true;
    for (const MoveKind& mk : s->moves) all_trn = all_trn && mk.type == MCG_MOVE_TRN;
    if (!trace && !follow && save_each == 0 && all_trn && h.cut == MCG_CUT_SWITCH && h.pbc != MCG_PBC_NONE &&
        h.prec == MCG_PREC_FP64 && !E.has_bonded_terms() && SingleEngine::replay_fits(s->moves) &&
        SingleEngine::replay_cluster_ok()) {
        rc = E.metropolis_device(gen, s->moves, beta, nsteps, &etot, &acc);
        if (rc) return rc;
        if (final_etot) *final_etot = etot;
        if (n_accepted) *n_accepted = acc;
        if (n_ties) *n_ties = 0;
        return MCG_OK;
    }
    std::vector<int> atoms;
    std::vector<double> nx, ny, nz;
    std::vector<double>& X = E.host_x;
    std::vector<double>& Y = E.host_y;
    std::vector<double>& Z = E.host_z;
    auto wrap = [&](double& v, int k) {
        if (h.pbc != MCG_PBC_NONE) {
            double t = h.rL[k] * v;
            double r = (double)(t >= 0. ? (int)(t + 0.5) : (int)(t - 0.5));
            v -= h.L[k] * r;
        }
    };
    for (int st = 1; st <= nsteps; st++) {
        int imvtyp = (int)(nmvtyp * dAlpha(gen));
        const MoveKind& mk = s->moves[imvtyp];
        int imvatm = (int)(mk.ninst() * dAlpha(gen));
        atoms.clear();
        for (int r = mk.rstart[imvatm]; r < mk.rstart[imvatm + 1]; r++)
            for (int a = mk.ranges[2 * r]; a <= mk.ranges[2 * r + 1]; a++) atoms.push_back(a);
        const int m = (int)atoms.size();
        nx.resize(m); ny.resize(m); nz.resize(m);
        for (int k = 0; k < m; k++) { nx[k] = X[atoms[k]]; ny[k] = Y[atoms[k]]; nz[k] = Z[atoms[k]]; }
        double rec[12] = {0};
        double r[3];
        auto sphere = [&]() {
            double rx, ry, rz;
            do { rx = dMove(gen); ry = dMove(gen); rz = dMove(gen); } while ((rx * rx + ry * ry + rz * rz) > 1.0);
            r[0] = rx; r[1] = ry; r[2] = rz;
        };
        double rang = 0.0;
        if (mk.type == MCG_MOVE_TRN) {
            sphere();
            r[0] *= dmax[imvtyp]; r[1] *= dmax[imvtyp]; r[2] *= dmax[imvtyp];
            rec[3] = r[0]; rec[4] = r[1]; rec[5] = r[2];
            for (int k = 0; k < m; k++) {
                nx[k] += r[0]; ny[k] += r[1]; nz[k] += r[2];
                wrap(nx[k], 0); wrap(ny[k], 1); wrap(nz[k], 2);
            }
        } else {
            sphere();
            rang = dmax[imvtyp] * dMove(gen);
            rec[3] = r[0]; rec[4] = r[1]; rec[5] = r[2];
            double mat[3][3] = {{1., 0., 0.}, {0., 1., 0.}, {0., 0., 1.}};
            double ang = rang * PI / 180.0;
            double rn = 1.0 / std::sqrt(r[0] * r[0] + r[1] * r[1] + r[2] * r[2]);
            double v[3] = {r[0] * rn, r[1] * rn, r[2] * rn};
            double T[3][3] = {{0., -v[2], v[1]}, {v[2], 0., -v[0]}, {-v[1], v[0], 0.}};
            double T2[3][3] = {{0., 0., 0.}, {0., 0., 0.}, {0., 0., 0.}};
            double v1 = std::sin(ang), v2 = 1.0 - std::cos(ang);
            for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++) mat[i][j] += T[i][j] * v1;
            for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++) for (int k = 0; k < 3; k++) T2[i][j] += T[i][k] * T[k][j];
            for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++) mat[i][j] += T2[i][j] * v2;
            double pv[3] = {0., 0., 0.};
            int piv = mk.pivot[imvatm];
            if (piv >= 0) { pv[0] = X[piv]; pv[1] = Y[piv]; pv[2] = Z[piv]; }
            else {
                double mt = 0.0;
                for (int k = 0; k < m; k++) {
                    double ms = h.mass[atoms[k]];
                    mt += ms; pv[0] += ms * nx[k]; pv[1] += ms * ny[k]; pv[2] += ms * nz[k];
                }
                pv[0] /= mt; pv[1] /= mt; pv[2] /= mt;
            }
            for (int k = 0; k < m; k++) {
                double px = nx[k] - pv[0], py = ny[k] - pv[1], pz = nz[k] - pv[2];
                nx[k] = pv[0] + mat[0][0] * px + mat[1][0] * py + mat[2][0] * pz;
                ny[k] = pv[1] + mat[0][1] * px + mat[1][1] * py + mat[2][1] * pz;
                nz[k] = pv[2] + mat[0][2] * px + mat[1][2] * py + mat[2][2] * pz;
                wrap(nx[k], 0); wrap(ny[k], 1); wrap(nz[k], 2);
            }
        }
        double de = 0.0;
        rc = E.delta_e(m, atoms.data(), nx.data(), ny.data(), nz.data(), &de);
        if (rc) return rc;
        double alpha = -1.0;
        bool accepted;
        if (de <= std::numeric_limits<double>::epsilon()) accepted = true;
        else { alpha = dAlpha(gen); accepted = alpha < std::exp(-beta * de); }
        if (follow) {
            bool want = follow[2 * (st - 1) + 1] != 0;
            if (follow[2 * (st - 1)] != imvtyp) return fail(MCG_EINVAL, "followed trace diverged at step " + std::to_string(st));
            if (want != accepted) {
                // only a tie may be overridden: the draw within 1e-6 of the acceptance threshold,
                // or (no draw) a dE within 1e-6 iu of the DBL_EPSILON bound
                const double margin = alpha >= 0.0 ? std::fabs(alpha - std::exp(-beta * de)) : std::fabs(de);
                if (!(margin <= 1e-6))
                    return fail(MCG_EINVAL, "followed decision differs at step " + std::to_string(st) +
                                                " and is not a tie (margin " + std::to_string(margin) + ")");
                ties++;
                accepted = want;
            }
        }
        double eold = etot;
        if (accepted) {
            rc = E.commit();
            if (rc) return rc;
            accTmp[imvtyp]++;
            etot += de;
            acc++;
        }
        for (int t = 0; t < nmvtyp; t++) {
            const MoveKind& mt = s->moves[t];
            if (mt.each != 0 && (st % mt.each) == 0) {  // MC::adjust_dmax, MC.cpp:165-173
                double ratio = (double)accTmp[t] / (double)mt.each;
                if (ratio > mt.target / 100) dmax[t] *= 1.10; else dmax[t] *= 0.9;
                accTmp[t] = 0;
            }
        }
        if (st % 50 == 0 && h.cut == MCG_CUT_SWITCH) {
            rc = E.update_lists();
            if (rc) return rc;
        }
        if (trace) {
            rec[0] = st; rec[1] = imvtyp; rec[2] = imvatm; rec[6] = rang; rec[7] = eold; rec[8] = eold + de;
            rec[9] = de; rec[10] = alpha; rec[11] = accepted ? 1.0 : 0.0;
            std::memcpy(trace + 12 * (size_t)(st - 1), rec, sizeof rec);
        }
        if (save_each > 0 && st % save_each == 0) {   // MC_metropolis.cpp:156-162
            const size_t k = (size_t)(st / save_each - 1);
            double* f = frames + k * 3 * (size_t)h.n;
            for (int a = 0; a < h.n; a++) { f[3 * a] = X[a]; f[3 * a + 1] = Y[a]; f[3 * a + 2] = Z[a]; }
            energies[k] = etot;
        }
    }
    if (final_etot) *final_etot = etot;
    if (n_accepted) *n_accepted = acc;
    if (n_ties) *n_ties = ties;
    return MCG_OK;
}

extern "C" {

int mcg_metropolis_run(mcg_system* s, int nsteps, uint64_t seed, int acceptance_units, double* trace,
                       const int* follow, double* final_etot, int64_t* n_accepted, int64_t* n_ties) {
    return metropolis_impl(s, nsteps, seed, acceptance_units, trace, follow, final_etot, n_accepted, n_ties, 0,
                           nullptr, nullptr);
}

int mcg_metropolis_run_saving(mcg_system* s, int nsteps, uint64_t seed, int acceptance_units, int save_each,
                              double* frames, double* energies, double* final_etot, int64_t* n_accepted) {
    if (save_each < 0) return fail(MCG_EINVAL, "save_each must be >= 0");
    if (save_each > 0 && nsteps >= save_each && (!frames || !energies)) return fail(MCG_EINVAL, "null frame or energy buffer");
    return metropolis_impl(s, nsteps, seed, acceptance_units, nullptr, nullptr, final_etot, n_accepted, nullptr,
                           save_each, frames, energies);
}

}  // extern "C"
