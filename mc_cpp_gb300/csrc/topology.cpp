// Host-side topology: system validation and unit conversion, exclusion / 1-4 lists, move
// instances.  One-time work per system; the result is uploaded to the device by the engines.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>

#include "engine.hpp"

namespace mcg {

static thread_local std::string g_err;
void set_error(const std::string& msg) { g_err = msg; }
int fail(int code, const std::string& msg) { g_err = msg; return code; }
const char* last_error_cstr() { return g_err.c_str(); }

int build_host_system(const mcg_system_desc* d, HostSystem& hs) {
    if (!d) return fail(MCG_EINVAL, "null system description");
    if (d->natom <= 0) return fail(MCG_EINVAL, "natom must be positive");
    if (!d->x || !d->y || !d->z || !d->q || !d->eps || !d->sig)
        return fail(MCG_EINVAL, "x, y, z, q, eps and sig are required");
    if (d->pbc_type < MCG_PBC_NONE || d->pbc_type > MCG_PBC_ORBIC) return fail(MCG_EINVAL, "bad pbc_type");
    if (d->cut_mode != MCG_CUT_FULL && d->cut_mode != MCG_CUT_SWITCH)
        return fail(MCG_EINVAL, "bad cut_mode (the reference implements full and switch only)");
    if (d->precision != MCG_PREC_FP64 && d->precision != MCG_PREC_MIXED) return fail(MCG_EINVAL, "bad precision");
    const int n = d->natom;
    hs.n = n;
    hs.pbc = d->pbc_type;
    // PerConditions::set_pbc_vectors (PerConditions.cpp:121-160): cubic copies a to b and c.
    if (hs.pbc == MCG_PBC_CUBIC) hs.L[0] = hs.L[1] = hs.L[2] = d->box[0];
    else if (hs.pbc == MCG_PBC_ORBIC) for (int k = 0; k < 3; k++) hs.L[k] = d->box[k];
    for (int k = 0; k < 3; k++) {
        if (hs.pbc != MCG_PBC_NONE && !(hs.L[k] > 0)) return fail(MCG_EINVAL, "box lengths must be positive");
        hs.rL[k] = hs.pbc != MCG_PBC_NONE ? 1.0 / hs.L[k] : 0.0;
    }
    hs.cut = d->cut_mode;
    hs.rc = d->cutoff; hs.ron = d->cuton; hs.dcut = d->dcut; hs.temp = d->temp;
    hs.prec = d->precision;
    if (hs.cut == MCG_CUT_SWITCH) {
        if (!(hs.rc > hs.ron) || !(hs.ron >= 0) || !(hs.dcut >= 0)) return fail(MCG_EINVAL, "need cutoff > cuton >= 0 and delta_cut >= 0");
        if (hs.pbc != MCG_PBC_NONE)
            for (int k = 0; k < 3; k++)
                if (hs.rc > 0.5 * hs.L[k]) return fail(MCG_EINVAL, "cutoff exceeds half the box (minimum image undefined)");
    }
    auto cp = [n](const double* src, std::vector<double>& dst, double dflt) {
        dst.resize(n);
        for (int i = 0; i < n; i++) dst[i] = src ? src[i] : dflt;
    };
    cp(d->x, hs.x, 0); cp(d->y, hs.y, 0); cp(d->z, hs.z, 0); cp(d->q, hs.q, 0);
    cp(d->sig, hs.sig, 0); cp(d->sig14, hs.sig14, 0); cp(d->mass, hs.mass, 1.0);
    if (d->param_units != MCG_UNITS_FILE && d->param_units != MCG_UNITS_INTERNAL) return fail(MCG_EINVAL, "bad param_units");
    const bool internal = d->param_units == MCG_UNITS_INTERNAL;
    const double kscale = internal ? 1.0 : KCALTOIU;   // x * 1.0 is exact: internal values pass unchanged
    hs.eps.resize(n); hs.eps14.resize(n);
    for (int i = 0; i < n; i++) {
        // IO_MDBAS.cpp:460,464: epsilon stored as sqrt(eps_file * kcaltoiu)
        if (d->eps[i] < 0 || (d->eps14 && d->eps14[i] < 0)) return fail(MCG_EINVAL, "negative epsilon");
        hs.eps[i] = internal ? d->eps[i] : std::sqrt(d->eps[i] * KCALTOIU);
        hs.eps14[i] = internal ? (d->eps14 ? d->eps14[i] : 0.0) : std::sqrt((d->eps14 ? d->eps14[i] : 0.0) * KCALTOIU);
        if (!std::isfinite(hs.x[i]) || !std::isfinite(hs.y[i]) || !std::isfinite(hs.z[i]))
            return fail(MCG_EINVAL, "non-finite coordinate at atom " + std::to_string(i));
    }
    hs.frozen.assign(n, 0);
    if (d->frozen) for (int i = 0; i < n; i++) hs.frozen[i] = d->frozen[i] ? 1 : 0;
    hs.resid.assign(n, 1);
    if (d->resid) for (int i = 0; i < n; i++) hs.resid[i] = d->resid[i];
    auto inrange = [n](int a) { return a >= 0 && a < n; };
    hs.bonds.clear(); hs.ubs.clear(); hs.angles.clear(); hs.dihes.clear(); hs.imprs.clear();
    for (int k = 0; k < d->nbond; k++) {
        int a = d->bond_atoms[2 * k], b = d->bond_atoms[2 * k + 1];
        if (!inrange(a) || !inrange(b)) return fail(MCG_EINVAL, "bond atom out of range");
        hs.bonds.push_back({a, b, d->bond_type ? d->bond_type[k] : 0, d->bond_k[k] * kscale, d->bond_r0[k],
                            d->bond_beta ? d->bond_beta[k] : 0.0});
    }
    for (int k = 0; k < d->nub; k++) {
        int a = d->ub_atoms[2 * k], b = d->ub_atoms[2 * k + 1];
        if (!inrange(a) || !inrange(b)) return fail(MCG_EINVAL, "Urey-Bradley atom out of range");
        hs.ubs.push_back({a, b, 0, d->ub_k[k] * kscale, d->ub_r0[k], 0.0});
    }
    for (int k = 0; k < d->nangle; k++) {
        const int* t = d->angle_atoms + 3 * k;
        if (!inrange(t[0]) || !inrange(t[1]) || !inrange(t[2])) return fail(MCG_EINVAL, "angle atom out of range");
        hs.angles.push_back({t[0], t[1], t[2], d->angle_type ? d->angle_type[k] : 0, d->angle_k[k] * kscale,
                             internal ? d->angle_theta0[k] : d->angle_theta0[k] * PI / 180.});
    }
    auto tors = [&](int cnt, const int* at, const int* ty, const int* ord, const double* kk, const double* ph,
                    const double* mu, std::vector<TorsT>& out) -> int {
        for (int k = 0; k < cnt; k++) {
            const int* t = at + 4 * k;
            for (int j = 0; j < 4; j++) if (!inrange(t[j])) return fail(MCG_EINVAL, "torsion atom out of range");
            out.push_back({t[0], t[1], t[2], t[3], ty ? ty[k] : 1, ord ? ord[k] : 1, kk[k] * kscale,
                           internal ? ph[k] : ph[k] * PI / 180., mu ? mu[k] : 1.0});
        }
        return MCG_OK;
    };
    int rc = tors(d->ndihe, d->dihe_atoms, d->dihe_type, d->dihe_order, d->dihe_k, d->dihe_phi0, d->dihe_mult, hs.dihes);
    if (rc) return rc;
    rc = tors(d->nimpr, d->impr_atoms, d->impr_type, d->impr_order, d->impr_k, d->impr_phi0, d->impr_mult, hs.imprs);
    if (rc) return rc;
    build_exclusions(hs);
    return MCG_OK;
}

namespace {
// Partner book of List_nonBonded's temporary arrays: per-atom partner lists in insertion order.
// A pair is recorded on both atoms unless the first atom already lists the second (the
// reference checks only row ii, List_nonBonded.cpp:230-240 and its repeats).
struct PartnerBook {
    std::vector<std::vector<int>> rows;
    std::vector<std::pair<int, int>> ver14;
    explicit PartnerBook(int n) : rows(n) {}
    bool has(int a, int b) const { return std::find(rows[a].begin(), rows[a].end(), b) != rows[a].end(); }
    void link(int a, int b) { rows[a].push_back(b); rows[b].push_back(a); }
    void add(int a, int b) { if (!has(a, b)) link(a, b); }
    void add14(int a, int b) { if (!has(a, b)) { ver14.emplace_back(a, b); link(a, b); } }
};
}  // namespace

void build_exclusions(HostSystem& hs) {
    const int n = hs.n;
    PartnerBook book(n);
    std::vector<std::vector<int>> graph(n);
    for (const BondT& b : hs.bonds) {               // excl_bonds: no duplicate check
        graph[b.a].push_back(b.b); graph[b.b].push_back(b.a);
        book.link(b.a, b.b);
    }
    for (const AngleT& a : hs.angles) { book.add(a.a, a.b); book.add(a.a, a.c); book.add(a.b, a.c); }
    for (const TorsT& t : hs.dihes) {               // a-d of a dihedral is a 1-4 candidate
        book.add(t.a, t.b); book.add(t.a, t.c); book.add14(t.a, t.d);
        book.add(t.b, t.c); book.add(t.b, t.d); book.add(t.c, t.d);
    }
    for (const TorsT& t : hs.imprs) {
        book.add(t.a, t.b); book.add(t.a, t.c); book.add(t.a, t.d);
        book.add(t.b, t.c); book.add(t.b, t.d); book.add(t.c, t.d);
    }
    for (int a = 0; a < n; a++)                       // excl_connectivity: 1-3 and 1-4 by bond walks
        for (int b : graph[a])
            for (int c : graph[b]) {
                if (c == a) continue;
                book.add(a, c);
                for (int d : graph[c]) if (d != a && d != b) book.add14(a, d);
            }
    // excl_final_Lists (List_nonBonded.cpp:705-775): keep partners within half the atom count
    // (forward) or the wrapped range (backward), sorted; then rotate the backward ones out of the
    // front of the row.  Only entries above i are ever matched by the consumers.
    const int half = n / 2, halfm1 = (n - 1) / 2;
    hs.exclStart.assign(n + 1, 0);
    hs.exclCount.assign(n, 0);
    hs.exclData.clear();
    hs.fexclStart.assign(n + 1, 0);
    hs.fexclCount.assign(n, 0);
    hs.fexclData.clear();
    hs.maxExclSpan = 0;
    std::vector<int> row;
    for (int i = 0; i < n; i++) {
        row.clear();
        for (int e : book.rows[i])
            if ((e > i && e - i < half) || (e < i && e - i + n < halfm1)) row.push_back(e);
        std::sort(row.begin(), row.end());
        const int c = (int)row.size();
        for (int pass = 0; pass < c; pass++)
            if (row[0] < i) for (int k = 0; k + 1 < c; k++) row[k] = row[k + 1];
        hs.exclStart[i] = (int)hs.exclData.size();
        hs.exclCount[i] = c;
        hs.exclData.insert(hs.exclData.end(), row.begin(), row.end());
        // full-mode cursor semantics: entries matched in order while strictly increasing above i
        hs.fexclStart[i] = (int)hs.fexclData.size();
        int prev = i;
        for (int k = 0; k < c; k++) {
            if (row[k] <= prev) break;
            hs.fexclData.push_back(row[k]);
            prev = row[k];
        }
        hs.fexclCount[i] = (int)hs.fexclData.size() - hs.fexclStart[i];
        for (int e : row) if (e > i) hs.maxExclSpan = std::max(hs.maxExclSpan, e - i);
    }
    hs.exclStart[n] = (int)hs.exclData.size();
    hs.fexclStart[n] = (int)hs.fexclData.size();
    hs.pairs14.clear();
    for (auto& p : book.ver14) { hs.pairs14.push_back(p.first); hs.pairs14.push_back(p.second); }
}

// List_Moves::gtrsfl (List_Moves.cpp:630-697): residue bounds of the residue holding `atom`,
// from consecutive 1-based global residue ids.
static bool residue_bounds(const HostSystem& hs, int atom, int& first, int& last) {
    const int n = hs.n;
    int nres = *std::max_element(hs.resid.begin(), hs.resid.end());
    if (nres < 1) return false;
    std::vector<int> resLast(nres + 1, n - 1);
    resLast[0] = -1;
    int cur = 1, idx = 0;
    for (int it = 0; it < n; it++)
        if (hs.resid[it] > cur) { cur++; if (idx + 1 <= nres) resLast[++idx] = it - 1; }
    resLast[nres] = n - 1;
    int lo = 1, hi = nres;
    while (lo <= hi) {
        int mid = (lo + hi) / 2;
        if (resLast[mid - 1] <= atom && resLast[mid] >= atom) { first = resLast[mid - 1] + 1; last = resLast[mid]; return true; }
        if (resLast[mid] <= atom) lo = mid + 1; else hi = mid - 1;
    }
    return false;
}

int build_move_kind(const HostSystem& hs, int type, int mode, const int* sele, double dmax, double target,
                    int each, MoveKind& mk) {
    const int n = hs.n;
    if (type != MCG_MOVE_TRN && type != MCG_MOVE_ROT) return fail(MCG_EINVAL, "move type must be TRN or ROT");
    if (mode < MCG_MODE_RESIDUE || mode > MCG_MODE_ATOM) return fail(MCG_EINVAL, "bad move mode");
    if (mode == MCG_MODE_ATOM && type == MCG_MOVE_ROT)
        return fail(MCG_EINVAL, "rotation with single atom mode is useless");  // List_Moves.cpp:284-289
    if (!sele) return fail(MCG_EINVAL, "null selection");
    mk = MoveKind();
    mk.type = type; mk.mode = mode; mk.dmax = dmax; mk.target = target; mk.each = each;
    mk.rstart.push_back(0);
    int nsel = 0;
    for (int i = 0; i < n; i++) nsel += sele[i] == 1;
    if (nsel == 0) return fail(MCG_EINVAL, "empty selection");
    std::vector<int> all;  // makeMoveList: maximal runs of selected atoms
    if (mode == MCG_MODE_ALL) {
        int prev = 0;
        for (int i = 0; i < n; i++) {
            if (prev == 0 && sele[i] >= 1) all.push_back(i);
            else if (prev >= 1 && sele[i] == 0) all.push_back(i - 1);
            prev = sele[i];
        }
        if (sele[n - 1] >= 1) all.push_back(n - 1);
    }
    const bool com = (mode == MCG_MODE_ALL && type == MCG_MOVE_ROT);  // centre-of-mass pivot
    for (int i = 0; i < n; i++) {
        if (sele[i] != 1 && !com) continue;
        if (mode == MCG_MODE_RESIDUE) {
            int a, b;
            if (!residue_bounds(hs, i, a, b)) return fail(MCG_EINVAL, "residue bounds not found (residue ids must be 1..R, consecutive)");
            mk.ranges.push_back(a); mk.ranges.push_back(b);
        } else if (mode == MCG_MODE_ALL) {
            mk.ranges.insert(mk.ranges.end(), all.begin(), all.end());
        } else {
            mk.ranges.push_back(i); mk.ranges.push_back(i);
        }
        mk.rstart.push_back((int)mk.ranges.size() / 2);
        if (type == MCG_MOVE_ROT) mk.pivot.push_back(com ? -1 : i);
        if (mode == MCG_MODE_ALL) break;
    }
    return MCG_OK;
}

}  // namespace mcg
