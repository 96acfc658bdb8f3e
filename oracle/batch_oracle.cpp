// batch_oracle — FP64 CPU restatement of one batched Monte Carlo chain, move by move.
//
// TEST INFRASTRUCTURE ONLY, like mc_oracle.cpp: only tests/ load it, as the checker of the
// batched sweep (mc_cpp_gb300/csrc/batch.cu).  The product never links, loads or runs it.
//
// One chain is a periodic box of identical rigid residues.  A trial move follows the reference's
// Metropolis step (MC_metropolis.cpp:80-133, apply_criterion :175-204) on residue TRN / ROT moves
// (Move.hpp:52-183, MOVE_TRN::translate_set and MOVE_ROT::rotate_set), with the random numbers of
// the batched engine: per chain a Philox4x32-10 stream (Salmon, Moraes, Dror, Shaw, "Parallel
// random numbers: as easy as 1, 2, 3", SC'11) whose counter is the move index.  Draw k of a chain
// is two Philox blocks, counters (k_lo, k_hi, chain, 0) and (k_lo, k_hi, chain, 1):
//
//   block 0: x -> move type (bit 0: rotation, when residues have more than one atom), y ->
//            residue (y * nres >> 32), z -> pivot atom (z * apr >> 32), w -> cos(theta) of the
//            direction (2u - 1);
//   block 1: x -> azimuth of the direction (2 pi u), y -> radius dmax * cbrt(u) (TRN) or angle
//            dmax * (2u - 1) degrees (ROT), z, w -> alpha = ((z << 21 ^ w >> 11) + 1) / 2^53;
//
// with u = (v >> 8) / 2^24.  The rotation turns the residue about its pivot atom using the
// minimum-image offset of each atom from the pivot (unit quaternion of half the angle).  Moved
// atoms are re-wrapped into the box.  dE is the FP64 sum of the reference's switched pair terms
// (FField_MDBAS.cpp:336-424 per pair, with Tools::distance2 and PerConditions::applyPBC) of the
// residue's atoms against every atom of the other residues, after minus before; every pair within
// the cutoff counts, so no neighbour list is involved.  The decision is the reference's
// criterion: accept when dE <= DBL_EPSILON, else when alpha < exp(-beta dE), beta in mol/kcal
// applied to dE in kcal/mol (physical units) or in iu (the reference's own units,
// MC_metropolis.cpp:188).  dmax is adjusted per move type as MC::adjust_dmax does
// (MC.cpp:165-173), capped.
//
// orcb_follow checks a sweep's per-move records against this restatement: for each record it
// draws the same move in FP64 and measures how far the recorded proposal lies from it, computes
// the FP64 dE of the recorded proposal and the FP64 decision, then applies the RECORDED decision
// and positions, so the restatement follows the device chain exactly and every move is checked
// against the state the device saw.
#include <cfloat>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

namespace {

#include "ref_math.hpp"

struct U4 { uint32_t x, y, z, w; };

// Philox4x32-10: ten rounds of the 4x32 S-box with multipliers 0xD2511F53, 0xCD9E8D57 and the
// Weyl key increments 0x9E3779B9, 0xBB67AE85 (the published constants).
U4 philox4x32_10(U4 c, uint32_t k0, uint32_t k1) {
    const uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u, W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
    for (int r = 0; r < 10; r++) {
        const uint64_t p0 = (uint64_t)M0 * c.x, p1 = (uint64_t)M1 * c.z;
        c = U4{(uint32_t)(p1 >> 32) ^ c.y ^ k0, (uint32_t)p1, (uint32_t)(p0 >> 32) ^ c.w ^ k1, (uint32_t)p0};
        k0 += W0;
        k1 += W1;
    }
    return c;
}

double u24(uint32_t v) { return (double)(v >> 8) * (1.0 / 16777216.0); }

// one record of a logged sweep: the layout of struct mcg_batch_move (include/mcg.h)
struct MoveRecord {
    double de;
    int residue, flags;
    uint32_t ahi, alo;
    double xyz[8][3];
};
static_assert(sizeof(MoveRecord) == 216, "layout of mcg_batch_move");

struct Chain {
    int n = 0, apr = 1, nres = 0, ntypes = 1;
    Pbc pbc;
    double rc = 12, ron = 10, beta = 0;
    std::vector<double> x, y, z, q, eps, sig;
    uint32_t key0 = 0, key1 = 0, chain = 0;
    double dmax[2] = {0, 0}, cap[2] = {0, 0}, target[2] = {0, 0};
    int each[2] = {0, 0}, acc_tmp[2] = {0, 0};
    uint64_t moves = 0;                          // Philox counter of the next move

    // Switched pair energy (iu) of atoms i (at p) and j, FField_MDBAS.cpp:336-424 for one pair.
    double pair(const double p[3], int i, int j) const {
        const double pj[3] = {x[j], y[j], z[j]};
        const double r2 = distance2(p, pj, pbc);
        const double c2 = rc * rc, n2 = ron * ron;
        if (r2 > c2) return 0.0;
        const double rt = 1. / sqrt(r2);
        double pe = q[i] * q[j] * rt;
        double pv = eps[i] * eps[j] * (X12<double>((sig[i] + sig[j]) * rt) - X6<double>((sig[i] + sig[j]) * rt));
        if (r2 > n2) {
            const double s1 = c2 - r2;
            const double sw = X2<double>(s1) * (c2 + 2. * r2 - 3. * n2) * (1. / X3<double>(c2 - n2));
            pe *= sw;
            pv *= sw;
        }
        return CHGCHARMM * KCALTOIU * pe + 4.0 * pv;
    }

    // dE of moving residue r to nxyz (apr x 3), against every atom of the other residues (the
    // atom loop split over OpenMP threads for large chains; FP64 sums, order-insensitive at the
    // tolerances this checks).
    double delta_e(int r, const double (*nxyz)[3]) const {
        double eold = 0.0, enew = 0.0;
        for (int k = 0; k < apr; k++) {
            const int a = r * apr + k;
            const double po[3] = {x[a], y[a], z[a]};
            const double pn[3] = {nxyz[k][0], nxyz[k][1], nxyz[k][2]};
#pragma omp parallel for reduction(+ : eold, enew) schedule(static) if (n > 8192)
            for (int b = 0; b < n; b++) {
                if (b / apr == r) continue;
                eold += pair(po, a, b);
                enew += pair(pn, a, b);
            }
        }
        return enew - eold;
    }

    double wrap(double v, int t) const { return v - pbc.L[t] * std::nearbyint(v * pbc.rL[t]); }

    // The move with Philox counter k, in FP64: residue, type, proposed positions, alpha.
    void propose(uint64_t k, int* res, int* rot, double (*nxyz)[3], double* alpha) const {
        const U4 q0 = philox4x32_10(U4{(uint32_t)k, (uint32_t)(k >> 32), chain, 0u}, key0, key1);
        const U4 q1 = philox4x32_10(U4{(uint32_t)k, (uint32_t)(k >> 32), chain, 1u}, key0, key1);
        const int r = (int)(((uint64_t)q0.y * (uint64_t)nres) >> 32);
        const bool ro = ntypes == 2 && (q0.x & 1u);
        const int piv = (int)(((uint64_t)q0.z * (uint64_t)apr) >> 32);
        const double ct = 2.0 * u24(q0.w) - 1.0, st = std::sqrt(std::fmax(0.0, 1.0 - ct * ct));
        const double phi = 2.0 * PI * u24(q1.x);
        const double u[3] = {st * std::cos(phi), st * std::sin(phi), ct};
        if (!ro) {
            const double rad = dmax[0] * std::cbrt(u24(q1.y));
            for (int j = 0; j < apr; j++) {
                const int a = r * apr + j;
                nxyz[j][0] = wrap(x[a] + rad * u[0], 0);
                nxyz[j][1] = wrap(y[a] + rad * u[1], 1);
                nxyz[j][2] = wrap(z[a] + rad * u[2], 2);
            }
        } else {
            const double half = dmax[1] * (2.0 * u24(q1.y) - 1.0) * PI / 360.0;
            const double qw = std::cos(half), qv[3] = {std::sin(half) * u[0], std::sin(half) * u[1], std::sin(half) * u[2]};
            const int p = r * apr + piv;
            const double pv[3] = {x[p], y[p], z[p]};
            for (int j = 0; j < apr; j++) {
                const int a = r * apr + j;
                const double pa[3] = {x[a], y[a], z[a]};
                double o[3];
                distance2(pv, pa, pbc, o);      // minimum-image offset of the atom from the pivot
                // o' = o + 2 qw (qv x o) + 2 qv x (qv x o)
                const double t[3] = {2.0 * (qv[1] * o[2] - qv[2] * o[1]), 2.0 * (qv[2] * o[0] - qv[0] * o[2]),
                                     2.0 * (qv[0] * o[1] - qv[1] * o[0])};
                const double d[3] = {qw * t[0] + (qv[1] * t[2] - qv[2] * t[1]), qw * t[1] + (qv[2] * t[0] - qv[0] * t[2]),
                                     qw * t[2] + (qv[0] * t[1] - qv[1] * t[0])};
                for (int c = 0; c < 3; c++) nxyz[j][c] = wrap(pa[c] + d[c], c);
            }
        }
        *res = r;
        *rot = ro ? 1 : 0;
        *alpha = ((double)(((uint64_t)q1.z << 21) ^ (uint64_t)(q1.w >> 11)) + 1.0) * (1.0 / 9007199254740992.0);
    }

    // MC_metropolis::apply_criterion, MC_metropolis.cpp:175-204
    bool accept(double de, double alpha) const {
        if (de <= DBL_EPSILON) return true;
        return alpha < std::exp(-beta * de);
    }

    // MC::adjust_dmax (MC.cpp:165-173) after a move, per type, capped
    void after_move(int rot, bool accepted) {
        if (accepted) acc_tmp[rot]++;
        moves++;
        for (int t = 0; t < 2; t++) {
            if (each[t] > 0 && moves % (uint64_t)each[t] == 0) {
                const double ratio = (double)acc_tmp[t] / (double)each[t];
                dmax[t] = std::fmin(cap[t], dmax[t] * (ratio > target[t] ? 1.10 : 0.9));
                acc_tmp[t] = 0;
            }
        }
    }
};

}  // namespace

extern "C" {

// One chain: natom atoms in residues of apr atoms; per-atom charge, file epsilon (kcal/mol; stored
// as sqrt(eps * 418.4), IO_MDBAS.cpp:460) and MDBAS half-sigma; periodic box L[3] (cubic or
// orthorhombic); switch rc / ron; temperature; acceptance_units 1 = physical (dE in kcal/mol),
// 0 = the reference's units; Philox key from the batch seed and the chain index exactly as the
// batched engine derives it; dmax (A, degrees), adjustment periods, targets (percent) and caps.
void* orcb_create(int natom, int apr, const double* L, const double* q, const double* eps_file, const double* sig,
                  double rc, double ron, double temp, int acceptance_units, uint64_t seed, int chain,
                  const double* dmax, const int* each, const double* target_pct, const double* cap) {
    if (natom <= 0 || apr <= 0 || apr > 8 || natom % apr) return nullptr;
    Chain* c = new Chain;
    c->n = natom;
    c->apr = apr;
    c->nres = natom / apr;
    c->ntypes = apr > 1 ? 2 : 1;
    c->pbc.type = PBC_ORBIC;
    for (int t = 0; t < 3; t++) { c->pbc.L[t] = L[t]; c->pbc.rL[t] = 1.0 / L[t]; }
    c->rc = rc;
    c->ron = ron;
    c->beta = 1.0 / ((RBOLTZUI / KCALTOIU) * temp);
    if (acceptance_units == 1) c->beta /= KCALTOIU;
    c->q.assign(q, q + natom);
    c->sig.assign(sig, sig + natom);
    c->eps.resize(natom);
    for (int i = 0; i < natom; i++) c->eps[i] = std::sqrt(eps_file[i] * KCALTOIU);
    c->x.assign(natom, 0.0); c->y.assign(natom, 0.0); c->z.assign(natom, 0.0);
    const uint64_t key = (seed + 1) * 0x9E3779B97F4A7C15ull ^ ((uint64_t)chain * 0xD1B54A32D192ED03ull);
    c->key0 = (uint32_t)key;
    c->key1 = (uint32_t)(key >> 32);
    c->chain = (uint32_t)chain;
    for (int t = 0; t < 2; t++) {
        c->dmax[t] = dmax[t];
        c->each[t] = each[t];
        c->target[t] = target_pct[t] / 100.0;
        c->cap[t] = cap[t];
    }
    return c;
}

void orcb_destroy(void* h) { delete (Chain*)h; }

void orcb_set_coords(void* h, const double* x, const double* y, const double* z) {
    Chain* c = (Chain*)h;
    std::memcpy(c->x.data(), x, sizeof(double) * c->n);
    std::memcpy(c->y.data(), y, sizeof(double) * c->n);
    std::memcpy(c->z.data(), z, sizeof(double) * c->n);
}

void orcb_get_coords(void* h, double* x, double* y, double* z) {
    Chain* c = (Chain*)h;
    std::memcpy(x, c->x.data(), sizeof(double) * c->n);
    std::memcpy(y, c->y.data(), sizeof(double) * c->n);
    std::memcpy(z, c->z.data(), sizeof(double) * c->n);
}

// One Philox4x32-10 block (known-answer checks of the restatement).
void orcb_philox(const uint32_t* ctr, const uint32_t* key, uint32_t* out) {
    const U4 r = philox4x32_10(U4{ctr[0], ctr[1], ctr[2], ctr[3]}, key[0], key[1]);
    out[0] = r.x; out[1] = r.y; out[2] = r.z; out[3] = r.w;
}

// Philox counter of the next move (the chain's trial count so far).
void orcb_set_moves(void* h, uint64_t moves) { ((Chain*)h)->moves = moves; }

void orcb_get_dmax(void* h, double* dmax) { dmax[0] = ((Chain*)h)->dmax[0]; dmax[1] = ((Chain*)h)->dmax[1]; }

// Total nonbonded energy (iu): every residue pair's atom pairs within the cutoff, FP64.
double orcb_energy(void* h) {
    const Chain* c = (const Chain*)h;
    double e = 0.0;
#pragma omp parallel for reduction(+ : e) schedule(dynamic, 64)
    for (int a = 0; a < c->n; a++) {
        const double pa[3] = {c->x[a], c->y[a], c->z[a]};
        for (int b = (a / c->apr + 1) * c->apr; b < c->n; b++) e += c->pair(pa, a, b);
    }
    return e;
}

// Follows nrec recorded moves (the chain's records of a logged sweep, in order) from the chain's
// current state and Philox counter.  Per record k it writes:
//   out[8k + 0]  1 when the recorded residue and move type are the ones the Philox draw gives
//   out[8k + 1]  largest distance (A) between a recorded and an FP64-proposed atom position
//   out[8k + 2]  the FP64 dE (iu) of the recorded proposal
//   out[8k + 3]  the FP64 decision on that dE (1 accept)
//   out[8k + 4]  the FP64 decision on the RECORDED dE (the device's criterion restated)
//   out[8k + 5]  alpha of the draw
//   out[8k + 6]  exp(-beta dE_FP64)
//   out[8k + 7]  1 when the recorded alpha words equal the draw's
// then applies the recorded decision and positions.
void orcb_follow(void* h, int nrec, const void* records, double* out) {
    Chain* c = (Chain*)h;
    const MoveRecord* rec = (const MoveRecord*)records;
    double nxyz[8][3];
    for (int k = 0; k < nrec; k++) {
        const MoveRecord& m = rec[k];
        int res = -1, rot = -1;
        double alpha = 0.0;
        c->propose(c->moves, &res, &rot, nxyz, &alpha);
        const U4 q1 = philox4x32_10(U4{(uint32_t)c->moves, (uint32_t)(c->moves >> 32), c->chain, 1u}, c->key0, c->key1);
        const int rrot = m.flags & 1;
        const bool racc = (m.flags & 2) != 0;
        double* o = out + 8 * (size_t)k;
        o[0] = (res == m.residue && rot == rrot) ? 1.0 : 0.0;
        const int r = m.residue;
        if (r < 0 || r >= c->nres) {            // a record outside the chain: flag it, change nothing
            o[0] = 0.0;
            for (int t = 1; t < 8; t++) o[t] = NAN;
            c->after_move(0, false);
            continue;
        }
        double err = 0.0;
        if (o[0] != 0.0)
            for (int j = 0; j < c->apr; j++) {
                double d[3];
                const double a[3] = {nxyz[j][0], nxyz[j][1], nxyz[j][2]}, b[3] = {m.xyz[j][0], m.xyz[j][1], m.xyz[j][2]};
                err = std::fmax(err, std::sqrt(distance2(a, b, c->pbc, d)));
            }
        o[1] = o[0] != 0.0 ? err : NAN;
        const double de = c->delta_e(r, m.xyz);
        o[2] = de;
        o[3] = c->accept(de, alpha) ? 1.0 : 0.0;
        const double ralpha = ((double)(((uint64_t)m.ahi << 21) ^ (uint64_t)(m.alo >> 11)) + 1.0) * (1.0 / 9007199254740992.0);
        o[4] = c->accept(m.de, ralpha) ? 1.0 : 0.0;
        o[5] = alpha;
        o[6] = std::exp(-c->beta * de);
        o[7] = (m.ahi == q1.z && m.alo == q1.w) ? 1.0 : 0.0;
        if (racc)
            for (int j = 0; j < c->apr; j++) {
                const int a = r * c->apr + j;
                c->x[a] = m.xyz[j][0]; c->y[a] = m.xyz[j][1]; c->z[a] = m.xyz[j][2];
            }
        c->after_move(rrot, racc);
    }
}

}  // extern "C"
