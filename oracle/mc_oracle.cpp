// mc_oracle — CPU restatement of FHedin/mc_cpp's nonbonded Monte Carlo energy path.
//
// TEST INFRASTRUCTURE ONLY.  Only tests/, __graft_entry__.smoke() and bench.py's cpu_baseline /
// --impl reference legs may load this library, and only as the checker or as the timed CPU
// baseline.  The product (mc_cpp_gb300) never links, loads or falls back to it.
//
// Parity pin: every function below restates a reference function (file:line in its comment) with
// the same operation order, built with -ffp-contract=off like the reference build in
// oracle/ref.mk, so FP64 results agree with the compiled reference bit for bit.  tests/golden/
// holds the reference's own outputs (energies, exclusion/1-4/Verlet rows, MC traces) and
// tests/test_oracle.py checks this file against them.
//
// Units follow the reference: energies in internal units (1 kcal/mol = 418.4 iu,
// Constants.hpp:29), per-atom epsilon stored as sqrt(eps_kcal * 418.4) (IO_MDBAS.cpp:460),
// sigma is the MDBAS half-sigma so a pair uses (sig_i + sig_j) (FField_MDBAS.cpp:333).
#include <cmath>
#include <cstdint>
#include <cstring>
#include <cfloat>
#include <limits>
#include <random>
#include <vector>
#include <algorithm>
#include <chrono>

namespace {

#include "ref_math.hpp"

enum { CUT_FULL = 0, CUT_SWITCH = 1 };
enum { MV_TRN = 1, MV_ROT = 2 };
enum { MODE_RESIDUE = 0, MODE_ALL = 1, MODE_ATOM = 2 };

struct Bond { int a, b, type; double k, r0, beta; };
struct Angle { int a, b, c, type; double k, theta0; };
struct Dihe { int a, b, c, d, type, order; double k, phi0, mult; };

struct MoveType {
    int type, mode;
    std::vector<std::vector<int>> inst;  // per instance: [ng, nn, first, last, ...] (List_Moves layout)
    std::vector<int> pivot;              // per instance pivot atom or -1 (ROT only)
    double dmax, target;
    int each;
};

struct Oracle {
    int n = 0;
    Pbc pbc;
    int cutMode = CUT_SWITCH;
    double cutoff = 12, cuton = 10, deltacut = 2;
    double temp = 300;
    std::vector<double> x, y, z, q, eps, sig, eps14, sig14, mass;
    std::vector<unsigned char> frozen;
    std::vector<int> resid;
    std::vector<Bond> bonds, ubs;
    std::vector<Angle> angles;
    std::vector<Dihe> dihes, imprs;
    // List_nonBonded state
    std::vector<int> exclPair;
    std::vector<std::vector<int>> exclList;
    std::vector<int> neighList14;
    int nPair14 = 0;
    std::vector<int> neighPair;
    std::vector<std::vector<int>> neighList;
    // energy components (FField.hpp:123-125)
    double tot = 0, pot = 0, kin = 0, elec = 0, vdw = 0, bond = 0, ang = 0, ub = 0, dihe = 0, impr = 0;
    std::vector<MoveType> moves;
    // 0: the reference's acceptance (beta in mol/kcal applied to dE in iu, MC_metropolis.cpp:188);
    // 1: physical (dE converted to kcal/mol).  Only the batched-workload CPU baseline sets 1.
    int acceptance_units = 0;

    inline void crd(int i, double d[3]) const { d[0] = x[i]; d[1] = y[i]; d[2] = z[i]; }

    // ---- exclusion lists: List_nonBonded.cpp:143-775 -------------------------------------
    // tempAtom rows are kept in insertion order; a pair is added to both rows unless already in
    // row ii (the reference's duplicate check scans row ii only).
    std::vector<std::vector<int>> tempAtom, tempConnect;
    std::vector<std::vector<int>> tempVer14;

    bool in_row(int ii, int jj) const {
        for (int v : tempAtom[ii]) if (v == jj) return true;
        return false;
    }
    void add_pair(int ii, int jj) { tempAtom[ii].push_back(jj); tempAtom[jj].push_back(ii); }
    void add_if_new(int ii, int jj) { if (!in_row(ii, jj)) add_pair(ii, jj); }

    void build_exclude_list() {
        tempAtom.assign(n, {});
        tempConnect.assign(n, {});
        tempVer14.clear();
        // excl_bonds :184-212 (no duplicate check)
        for (const Bond& b : bonds) {
            tempConnect[b.a].push_back(b.b);
            tempConnect[b.b].push_back(b.a);
            add_pair(b.a, b.b);
        }
        // excl_angles :214-291
        for (const Angle& a : angles) {
            add_if_new(a.a, a.b);
            add_if_new(a.a, a.c);
            add_if_new(a.b, a.c);
        }
        // excl_dihedrals :293-427 (the a-d pair becomes a 1-4 pair when new)
        for (const Dihe& d : dihes) {
            add_if_new(d.a, d.b);
            add_if_new(d.a, d.c);
            if (!in_row(d.a, d.d)) { tempVer14.push_back({d.a, d.d}); add_pair(d.a, d.d); }
            add_if_new(d.b, d.c);
            add_if_new(d.b, d.d);
            add_if_new(d.c, d.d);
        }
        // excl_impropers :429-565
        for (const Dihe& d : imprs) {
            add_if_new(d.a, d.b);
            add_if_new(d.a, d.c);
            add_if_new(d.a, d.d);
            add_if_new(d.b, d.c);
            add_if_new(d.b, d.d);
            add_if_new(d.c, d.d);
        }
        // excl_connectivity :567-703
        for (int ia = 0; ia < n; ia++) {
            for (size_t j = 0; j < tempConnect[ia].size(); j++) {
                int ib = tempConnect[ia][j];
                for (size_t k = 0; k < tempConnect[ib].size(); k++) {
                    int ic = tempConnect[ib][k];
                    if (ic == ia) continue;
                    add_if_new(ia, ic);
                    for (size_t l = 0; l < tempConnect[ic].size(); l++) {
                        int id = tempConnect[ic][l];
                        if (id == ia || id == ib) continue;
                        if (!in_row(ia, id)) { tempVer14.push_back({ia, id}); add_pair(ia, id); }
                    }
                }
            }
        }
        // excl_final_Lists :705-775
        const int hnAtom = n / 2, hm1nAtom = (n - 1) / 2;
        exclPair.assign(n, 0);
        exclList.assign(n, {});
        for (int i = 0; i < n; i++) {
            std::vector<int>& row = exclList[i];
            row.assign(tempAtom[i].size(), 0);
            int jj = 0;
            for (size_t j = 0; j < tempAtom[i].size(); j++) {
                int e = tempAtom[i][j];
                if (((e > i) && ((e - i) < hnAtom)) || ((e < i) && ((e - i + n) < hm1nAtom))) {
                    row[jj] = e;
                    for (int k = jj; k > 0; k--)  // insertion sort step :729-740
                        if (row[k] < row[k - 1]) std::swap(row[k], row[k - 1]);
                    jj++;
                }
            }
            exclPair[i] = jj;
        }
        // wrap rotation :749-766.  The reference also writes the rotated entry at index
        // exclPair[i], one past the used part of the row; nothing reads it, so it is not kept.
        for (int i = 0; i < n; i++) {
            std::vector<int>& row = exclList[i];
            for (int jj = 0; jj < exclPair[i]; jj++) {
                if (row[0] < i) {
                    for (int kk = 0; kk < exclPair[i] - 1; kk++) row[kk] = row[kk + 1];
                }
            }
        }
        nPair14 = (int)tempVer14.size();
        neighList14.assign(2 * nPair14, 0);
        for (int i = 0; i < nPair14; i++) { neighList14[2 * i] = tempVer14[i][0]; neighList14[2 * i + 1] = tempVer14[i][1]; }
        tempAtom.clear(); tempConnect.clear(); tempVer14.clear();
    }

    // ---- Verlet list: List_nonBonded.cpp:836-915 (update_verlet_list) --------------------
    void update_verlet_list() {
        double cutnb2 = cutoff + deltacut;
        cutnb2 *= cutnb2;
        neighPair.assign(n, 0);
        neighList.assign(n, {});
#pragma omp parallel for schedule(dynamic, 16)
        for (int i = 0; i < n; i++) {
            double di[3], dj[3];
            crd(i, di);
            std::vector<int>& row = neighList[i];
            for (int j = i + 1; j < n; j++) {
                crd(j, dj);
                double r2 = distance2(di, dj, pbc);
                if (r2 <= cutnb2) {
                    int exclude = 0;
                    if (frozen[i] && frozen[j]) exclude = 1;
                    else
                        for (int k = 0; k < exclPair[i]; k++)
                            if (exclList[i][k] == j) { exclude = 1; break; }
                    if (!exclude) row.push_back(j);
                }
            }
            neighPair[i] = (int)row.size();
        }
    }

    void build_lists() {
        build_exclude_list();
        if (cutMode != CUT_FULL) update_verlet_list();
    }

    // ---- energies: FField_MDBAS.cpp -------------------------------------------------------
    static inline double eelec(double qi, double qj, double rt) { return qi * qj * rt; }  // :321-325
    static inline double evdw(double ei, double ej, double si, double sj, double rt) {   // :328-334
        return ei * ej * (X12<double>((si + sj) * rt) - X6<double>((si + sj) * rt));
    }

    void nonbonded_full() {  // :194-265
        double lelec = 0., lvdw = 0.;
        double di[3], dj[3];
        for (int i = 0; i < n - 1; i++) {
            crd(i, di);
            double qi = q[i], epsi = eps[i], sigi = sig[i];
            int k = 0;
            for (int j = i + 1; j < n; j++) {
                bool exclude = false;
                if ((exclPair[i] > 0) && (exclList[i][k] == j)) {
                    exclude = true;
                    k++;
                    if (k >= exclPair[i]) k = exclPair[i] - 1;
                }
                if (!exclude) {
                    crd(j, dj);
                    double rt = distance2(di, dj, pbc);
                    rt = sqrt(rt);
                    rt = 1. / rt;
                    double pelec = eelec(qi, q[j], rt);
                    double pvdw = evdw(epsi, eps[j], sigi, sig[j], rt);
                    lelec += pelec;
                    lvdw += pvdw;
                }
            }
        }
        elec = CHGCHARMM * KCALTOIU * lelec;
        vdw = 4.0 * lvdw;
    }

    void nonbonded14() {  // :267-318
        double lelec = 0., levdw = 0.;
        double di[3], dj[3];
        for (int k = 0; k < nPair14; k++) {
            int i = neighList14[2 * k], j = neighList14[2 * k + 1];
            crd(i, di); crd(j, dj);
            double r2 = distance2(di, dj, pbc);
            double r = sqrt(r2);
            double rt = 1. / r;
            lelec += eelec(q[i], q[j], rt);
            levdw += evdw(eps14[i], eps14[j], sig14[i], sig14[j], rt);
        }
        elec += CHGCHARMM * KCALTOIU * lelec;
        vdw += 4.0 * levdw;
    }

    void nonbonded_switch() {  // :336-424
        double lelec = 0., levdw = 0.;
        const double ctoff2 = cutoff * cutoff, cton2 = cuton * cuton;
        const double switch2 = 1. / (X3<double>(ctoff2 - cton2));
        double di[3], dj[3];
        for (int i = 0; i < n; i++) {
            crd(i, di);
            double qi = q[i], epsi = eps[i], sigi = sig[i];
            for (int k = 0; k < neighPair[i]; k++) {
                int j = neighList[i][k];
                crd(j, dj);
                double r2 = distance2(di, dj, pbc);
                if (r2 <= ctoff2) {
                    double r = sqrt(r2);
                    double rt = 1. / r;
                    double pelec = eelec(qi, q[j], rt);
                    double pvdw = evdw(epsi, eps[j], sigi, sig[j], rt);
                    double sw = 1.0;
                    if (r2 > cton2) {
                        double s1 = ctoff2 - r2;
                        sw = X2<double>(s1) * (ctoff2 + 2. * r2 - 3. * cton2) * switch2;
                    }
                    pelec *= sw;
                    pvdw *= sw;
                    lelec += pelec;
                    levdw += pvdw;
                }
            }
        }
        elec = CHGCHARMM * KCALTOIU * lelec;
        vdw = 4.0 * levdw;
    }

    void nonbonded14_switch() {  // :426-488
        double lelec = 0., levdw = 0.;
        const double ctoff2 = cutoff * cutoff, cton2 = cuton * cuton;
        const double switch2 = 1. / (X3<double>(ctoff2 - cton2));
        double di[3], dj[3];
        for (int k = 0; k < nPair14; k++) {
            int i = neighList14[2 * k], j = neighList14[2 * k + 1];
            crd(i, di); crd(j, dj);
            double r2 = distance2(di, dj, pbc);
            double r = sqrt(r2);
            double rt = 1. / r;
            if (r2 <= ctoff2) {
                double pelec = eelec(q[i], q[j], rt);
                double pvdw = evdw(eps14[i], eps14[j], sig14[i], sig14[j], rt);
                double sw = 1.0;
                if (r2 > cton2) {
                    double s1 = ctoff2 - r2;
                    sw = X2<double>(s1) * (ctoff2 + 2. * r2 - 3. * cton2) * switch2;
                }
                pelec *= sw;
                pvdw *= sw;
                lelec += pelec;
                levdw += pvdw;
            }
        }
        elec += CHGCHARMM * KCALTOIU * lelec;
        vdw += 4.0 * levdw;
    }

    void ebond() {  // :490-534 (0 = harmonic, 1 = Morse, other = harmonic)
        double e = 0.0, di[3], dj[3];
        for (const Bond& b : bonds) {
            crd(b.a, di); crd(b.b, dj);
            double d = sqrt(distance2(di, dj, pbc));
            if (b.type == 1) {
                double ma = exp(-b.beta * (d - b.r0));
                double mb = X2<double>(ma);
                e += b.k * (mb - 2. * ma) + b.k;
            } else {
                e += 0.5 * b.k * X2<double>(d - b.r0);
            }
        }
        bond = e;
    }

    void eang() {  // :536-575
        double e = 0.0, di[3], dj[3], dk[3], dab[3], dbc[3];
        for (const Angle& a : angles) {
            crd(a.a, di); crd(a.b, dj); crd(a.c, dk);
            double rab = sqrt(distance2(di, dj, pbc, dab));
            double rbc = sqrt(distance2(dk, dj, pbc, dbc));
            double cost = (dab[0] * dbc[0] + dab[1] * dbc[1] + dab[2] * dbc[2]) / (rab * rbc);
            double theta = acos(cost);
            e += 0.5 * a.k * X2<double>(theta - a.theta0);
        }
        ang = e;
    }

    void eub() {  // :577-601
        double e = 0.0, di[3], dj[3];
        for (const Bond& b : ubs) {
            crd(b.a, di); crd(b.b, dj);
            double d = sqrt(distance2(di, dj, pbc));
            e += 0.5 * b.k * X2<double>(d - b.r0);
        }
        ub = e;
    }

    double torsions(const std::vector<Dihe>& list) const {  // :603-694 and :696-786
        double e = 0.;
        double di[3], dj[3], dk[3], dl[3], dab[3], dbc[3], dcd[3], pb[3], pc[3];
        for (const Dihe& t : list) {
            crd(t.a, di); crd(t.b, dj); crd(t.c, dk); crd(t.d, dl);
            dab[0] = di[0] - dj[0]; dab[1] = di[1] - dj[1]; dab[2] = di[2] - dj[2];  // vec_substract(dj, di, dab)
            pbc.apply(dab);
            double rbc = sqrt(distance2(dk, dj, pbc, dbc));
            dcd[0] = dk[0] - dl[0]; dcd[1] = dk[1] - dl[1]; dcd[2] = dk[2] - dl[2];  // vec_substract(dl, dk, dcd)
            pbc.apply(dcd);
            pb[0] = dab[1] * dbc[2] - dab[2] * dbc[1];
            pb[1] = dab[2] * dbc[0] - dab[0] * dbc[2];
            pb[2] = dab[0] * dbc[1] - dab[1] * dbc[0];
            double r2pb = X2<double>(pb[0]) + X2<double>(pb[1]) + X2<double>(pb[2]);
            double rpb = sqrt(r2pb);
            pc[0] = dbc[1] * dcd[2] - dbc[2] * dcd[1];
            pc[1] = dbc[2] * dcd[0] - dbc[0] * dcd[2];
            pc[2] = dbc[0] * dcd[1] - dbc[1] * dcd[0];
            double r2pc = X2<double>(pc[0]) + X2<double>(pc[1]) + X2<double>(pc[2]);
            double rpc = sqrt(r2pc);
            double pbpc = pb[0] * pc[0] + pb[1] * pc[1] + pb[2] * pc[2];
            double cosp = pbpc / (rpb * rpc);
            double sinp = (dbc[0] * (pc[1] * pb[2] - pc[2] * pb[1]) + dbc[1] * (pb[0] * pc[2] - pb[2] * pc[0]) +
                           dbc[2] * (pc[0] * pb[1] - pc[1] * pb[0])) / (rpb * rpc * rbc);
            double phi = atan2(sinp, cosp);
            if (t.type == 2) {  // DHARM
                phi = phi - t.phi0;
                phi = phi - ref_rint(phi / TWOPI) * TWOPI;
                e += 0.5 * t.k * (phi * phi);
            } else {            // DCOS and default
                e += t.k * (1. + cos(t.mult * phi - t.phi0));
            }
        }
        return e;
    }

    double getE() {  // FField_MDBAS::getE / getEtot / getEswitch, :53-192
        if (cutMode == CUT_FULL) { nonbonded_full(); nonbonded14(); }
        else { nonbonded_switch(); nonbonded14_switch(); }
        if (!bonds.empty()) ebond();
        if (!angles.empty()) eang();
        if (!ubs.empty()) eub();
        if (!dihes.empty()) dihe = torsions(dihes);
        if (!imprs.empty()) impr = torsions(imprs);
        pot = elec + vdw + bond + ang + ub + dihe + impr;
        tot = pot + kin;
        return tot;
    }

    // ---- moves: List_Moves.cpp:257-457,630-697; Move.hpp:42-183 ---------------------------
    // gtrsfl, List_Moves.cpp:630-697: residue [a1,a2] containing atom idx (residue ids 1..R).
    bool gtrsfl(int atomidx, int& a1, int& a2) const {
        int iresl = *std::max_element(resid.begin(), resid.end());
        std::vector<int> resLast(iresl + 1, 0);
        resLast[0] = -1;
        int last = 1, idx = 0;
        for (int it = 0; it < n; it++)
            if (resid[it] > last) { last++; if (idx + 1 <= iresl) resLast[++idx] = it - 1; }
        resLast[iresl] = n - 1;
        int iresf = 1;
        while (iresf <= iresl) {
            int mid = (iresl + iresf) / 2;
            if (resLast[mid - 1] <= atomidx && resLast[mid] >= atomidx) { a1 = resLast[mid - 1] + 1; a2 = resLast[mid]; return true; }
            else if (resLast[mid] <= atomidx) iresf = mid + 1;
            else iresl = mid - 1;
        }
        return false;
    }

    int add_move(int type, int mode, const int* sele, double dmax, double target, int each) {
        MoveType mv{type, mode, {}, {}, dmax, target, each};
        int nsel = 0;
        for (int i = 0; i < n; i++) nsel += sele[i] == 1;
        if (nsel == 0) return -1;
        if (mode == MODE_ATOM && type == MV_ROT) return -20;
        bool cofmas = false;
        std::vector<int> listp;
        if (mode == MODE_ALL) {  // makeMoveList :590-628
            int npair = 0, iprev = 0;
            for (int i = 0; i < n; i++) { if (iprev == 0 && sele[i] >= 1) npair++; iprev = sele[i]; }
            int nn = 2 * npair + 2;
            listp.assign(nn, 0);
            listp[0] = 1; listp[1] = nn - 1;
            int j = 2; iprev = 0;
            for (int i = 0; i < n; i++) {
                if (iprev == 0 && sele[i] >= 1) listp[j++] = i;
                else if (iprev >= 1 && sele[i] == 0) listp[j++] = i - 1;
                iprev = sele[i];
            }
            if (sele[n - 1] >= 1) listp[j] = n - 1;
            if (type == MV_ROT) cofmas = true;
        }
        for (int i = 0; i < n; i++) {
            if (sele[i] == 1 || cofmas) {
                if (mode == MODE_RESIDUE) {
                    int a1, a2;
                    if (!gtrsfl(i, a1, a2)) return -16;
                    mv.inst.push_back({1, 3, a1, a2});
                } else if (mode == MODE_ALL) {
                    mv.inst.push_back(listp);
                } else {
                    mv.inst.push_back({1, 3, i, i});
                }
                if (type == MV_ROT) mv.pivot.push_back(cofmas ? -1 : i);
                if ((mode == MODE_ALL && type == MV_TRN) || cofmas) break;
            }
        }
        moves.push_back(mv);
        return (int)moves.size() - 1;
    }

    template <typename F> static void for_ranges(const std::vector<int>& l, F f) {
        int ng = l[0], endng = ng + 2;
        for (int it1 = 1; it1 <= ng; it1++) {
            int nn = l[it1];
            for (int it2 = endng; it2 <= nn; it2 += 2) f(l[it2 - 1], l[it2]);
            endng = nn + 2;
        }
    }

    void wrap_atom(int i) {  // applyPBC(double&, double&, double&), PerConditions.cpp:258-277
        double d[3] = {x[i], y[i], z[i]};
        pbc.apply(d);
        x[i] = d[0]; y[i] = d[1]; z[i] = d[2];
    }

    void translate(const std::vector<int>& l, double r[3]) {  // MOVE_TRN::translate_set
        for_ranges(l, [&](int a, int b) {
            for (int i = a; i <= b; i++) { x[i] += r[0]; y[i] += r[1]; z[i] += r[2]; wrap_atom(i); }
        });
    }

    void rotate(const std::vector<int>& l, int pivot, double angle, double vec[3]) {  // MOVE_ROT::rotate_set
        double mat[3][3] = {{1., 0., 0.}, {0., 1., 0.}, {0., 0., 1.}};
        double angleRad = angle * PI / 180.0;
        double rn = 1.0 / sqrt(vec[0] * vec[0] + vec[1] * vec[1] + vec[2] * vec[2]);
        vec[0] *= rn; vec[1] *= rn; vec[2] *= rn;
        double T[3][3], T2[3][3] = {{0., 0., 0.}, {0., 0., 0.}, {0., 0., 0.}};
        T[0][0] = T[1][1] = T[2][2] = 0.0;
        T[2][1] = vec[0]; T[1][2] = -vec[0];
        T[0][2] = vec[1]; T[2][0] = -vec[1];
        T[1][0] = vec[2]; T[0][1] = -vec[2];
        double v1 = sin(angleRad), v2 = 1.0 - cos(angleRad);
        for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++) mat[i][j] += T[i][j] * v1;
        for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++) for (int k = 0; k < 3; k++) T2[i][j] += T[i][k] * T[k][j];
        for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++) mat[i][j] += T2[i][j] * v2;
        double pv[3] = {0., 0., 0.};
        if (pivot >= 0) crd(pivot, pv);
        else {  // Tools::getCentreOfMass(at_List, moveAtomList, cmass), Tools.hpp:112-147
            double mtot = 0.0;
            for_ranges(l, [&](int a, int b) {
                for (int i = a; i <= b; i++) { double m = mass[i]; mtot += m; pv[0] += m * x[i]; pv[1] += m * y[i]; pv[2] += m * z[i]; }
            });
            pv[0] /= mtot; pv[1] /= mtot; pv[2] /= mtot;
        }
        for_ranges(l, [&](int a, int b) {
            for (int i = a; i <= b; i++) {
                double px = x[i] - pv[0], py = y[i] - pv[1], pz = z[i] - pv[2];
                x[i] = pv[0] + mat[0][0] * px + mat[1][0] * py + mat[2][0] * pz;
                y[i] = pv[1] + mat[0][1] * px + mat[1][1] * py + mat[2][1] * pz;
                z[i] = pv[2] + mat[0][2] * px + mat[1][2] * py + mat[2][2] * pz;
                wrap_atom(i);
            }
        });
    }

    // MC_metropolis::run, MC_metropolis.cpp:45-173, with MC.cpp:110-173 for the draws.
    // trace (may be null): 12 doubles per step, the record layout of oracle/ref_probe.cpp.
    int mc_run(int nsteps, uint64_t seed, double* trace, double* final_etot, long long* n_acc) {
        const int nmvtyp = (int)moves.size();
        if (nmvtyp == 0) return -30;
        std::mt19937 gen;
        gen.seed(seed);
        std::uniform_real_distribution<double> dAlpha(0.0, 1.0), dMove(-1.0, 1.0);
        auto U = [&]() { return dAlpha(gen); };
        auto M = [&]() { return dMove(gen); };
        std::vector<double> dmax(nmvtyp);
        for (int t = 0; t < nmvtyp; t++) dmax[t] = moves[t].dmax;
        std::vector<int> accTmp(nmvtyp, 0);
        std::vector<double> bx(n), by(n), bz(n);
        double beta = 1.0 / ((RBOLTZUI / KCALTOIU) * temp);
        if (acceptance_units == 1) beta /= KCALTOIU;
        double etot = getE();
        long long acc = 0;
        for (int st = 1; st <= nsteps; st++) {
            double rec[12] = {0};
            int imvtyp = (int)(nmvtyp * U());
            const MoveType& mv = moves[imvtyp];
            int imvatm = (int)((int)mv.inst.size() * U());
            const std::vector<int>& l = mv.inst[imvatm];
            double eold = getE();
            for_ranges(l, [&](int a, int b) { for (int i = a; i <= b; i++) { bx[i] = x[i]; by[i] = y[i]; bz[i] = z[i]; } });
            double r[3], rang = 0.0;
            auto sphere = [&]() {  // MC::rndSphere :142-156
                double rx, ry, rz;
                do { rx = M(); ry = M(); rz = M(); } while ((rx * rx + ry * ry + rz * rz) > 1.0);
                r[0] = rx; r[1] = ry; r[2] = rz;
            };
            if (mv.type == MV_TRN) {
                sphere();
                r[0] *= dmax[imvtyp]; r[1] *= dmax[imvtyp]; r[2] *= dmax[imvtyp];
                rec[3] = r[0]; rec[4] = r[1]; rec[5] = r[2];
                translate(l, r);
            } else {
                sphere();
                rang = dmax[imvtyp] * M();
                rec[3] = r[0]; rec[4] = r[1]; rec[5] = r[2];
                rotate(l, mv.pivot[imvatm], rang, r);
            }
            double enew = getE();
            double de = enew - eold;
            bool accepted;
            double alpha = -1.0;
            if (de <= std::numeric_limits<double>::epsilon()) accepted = true;  // apply_criterion :175-204
            else { alpha = U(); accepted = alpha < exp(-beta * de); }
            if (accepted) { accTmp[imvtyp]++; etot += de; acc++; }
            else for_ranges(l, [&](int a, int b) { for (int i = a; i <= b; i++) { x[i] = bx[i]; y[i] = by[i]; z[i] = bz[i]; } });
            for (int t = 0; t < nmvtyp; t++) {
                if (moves[t].each != 0 && (st % moves[t].each) == 0) {  // MC::adjust_dmax :165-173
                    double ratio = (double)accTmp[t] / (double)moves[t].each;
                    if (ratio > moves[t].target / 100) dmax[t] *= 1.10; else dmax[t] *= 0.9;
                    accTmp[t] = 0;
                }
            }
            if (st % 50 == 0 && cutMode != CUT_FULL) update_verlet_list();
            if (trace) {
                rec[0] = st; rec[1] = imvtyp; rec[2] = imvatm; rec[6] = rang; rec[7] = eold; rec[8] = enew;
                rec[9] = de; rec[10] = alpha; rec[11] = accepted ? 1.0 : 0.0;
                memcpy(trace + 12 * (size_t)(st - 1), rec, sizeof rec);
            }
        }
        if (final_etot) *final_etot = etot;
        if (n_acc) *n_acc = acc;
        return 0;
    }
};

}  // namespace

extern "C" {

void* orc_create(int natom, int pbc_type, double a, double b, double c, int cut_mode, double cutoff,
                 double cuton, double deltacut, double temp) {
    Oracle* o = new Oracle;
    o->n = natom;
    o->pbc.type = pbc_type;
    if (pbc_type == PBC_CUBIC) { o->pbc.L[0] = o->pbc.L[1] = o->pbc.L[2] = a; }  // set_pbc_vectors :121-160
    else if (pbc_type == PBC_ORBIC) { o->pbc.L[0] = a; o->pbc.L[1] = b; o->pbc.L[2] = c; }
    for (int k = 0; k < 3; k++) o->pbc.rL[k] = (pbc_type != PBC_NONE) ? 1.0 / o->pbc.L[k] : 0.0;
    o->cutMode = cut_mode;
    o->cutoff = cutoff; o->cuton = cuton; o->deltacut = deltacut;
    o->temp = temp;
    o->x.assign(natom, 0); o->y.assign(natom, 0); o->z.assign(natom, 0);
    o->q.assign(natom, 0); o->eps.assign(natom, 0); o->sig.assign(natom, 0);
    o->eps14.assign(natom, 0); o->sig14.assign(natom, 0); o->mass.assign(natom, 1);
    o->frozen.assign(natom, 0); o->resid.assign(natom, 1);
    return o;
}

void orc_destroy(void* h) { delete (Oracle*)h; }

// eps_file / eps14_file are the forcefield file's epsilon columns (kcal/mol); stored as
// sqrt(eps * 418.4) exactly as IO_MDBAS::read_ff does (IO_MDBAS.cpp:460,464).
void orc_set_atoms(void* h, const double* x, const double* y, const double* z, const double* q,
                   const double* eps_file, const double* sig, const double* eps14_file, const double* sig14,
                   const double* mass, const unsigned char* frozen, const int* resid) {
    Oracle* o = (Oracle*)h;
    for (int i = 0; i < o->n; i++) {
        o->x[i] = x[i]; o->y[i] = y[i]; o->z[i] = z[i]; o->q[i] = q[i];
        o->eps[i] = sqrt(eps_file[i] * KCALTOIU); o->sig[i] = sig[i];
        o->eps14[i] = sqrt(eps14_file[i] * KCALTOIU); o->sig14[i] = sig14[i];
        if (mass) o->mass[i] = mass[i];
        if (frozen) o->frozen[i] = frozen[i];
        if (resid) o->resid[i] = resid[i];
    }
}

void orc_set_coords(void* h, const double* x, const double* y, const double* z) {
    Oracle* o = (Oracle*)h;
    for (int i = 0; i < o->n; i++) { o->x[i] = x[i]; o->y[i] = y[i]; o->z[i] = z[i]; }
}

void orc_get_coords(void* h, double* x, double* y, double* z) {
    Oracle* o = (Oracle*)h;
    for (int i = 0; i < o->n; i++) { x[i] = o->x[i]; y[i] = o->y[i]; z[i] = o->z[i]; }
}

// Bonded terms in file units (IO_MDBAS.cpp:186-443): k * 418.4, angles in degrees.
void orc_set_bonds(void* h, int nb, const int* ab, const int* type, const double* k, const double* r0, const double* beta) {
    Oracle* o = (Oracle*)h;
    o->bonds.clear();
    for (int i = 0; i < nb; i++) o->bonds.push_back({ab[2 * i], ab[2 * i + 1], type[i], k[i] * KCALTOIU, r0[i], beta[i]});
}
void orc_set_ub(void* h, int nb, const int* ab, const double* k, const double* r0) {
    Oracle* o = (Oracle*)h;
    o->ubs.clear();
    for (int i = 0; i < nb; i++) o->ubs.push_back({ab[2 * i], ab[2 * i + 1], 0, k[i] * KCALTOIU, r0[i], 0.0});
}
void orc_set_angles(void* h, int na, const int* abc, const int* type, const double* k, const double* theta0_deg) {
    Oracle* o = (Oracle*)h;
    o->angles.clear();
    for (int i = 0; i < na; i++)
        o->angles.push_back({abc[3 * i], abc[3 * i + 1], abc[3 * i + 2], type[i], k[i] * KCALTOIU, theta0_deg[i] * PI / 180.});
}
static void set_torsions(std::vector<Dihe>& out, int nd, const int* abcd, const int* type, const int* order,
                         const double* k, const double* phi0_deg, const double* mult) {
    out.clear();
    for (int i = 0; i < nd; i++)
        out.push_back({abcd[4 * i], abcd[4 * i + 1], abcd[4 * i + 2], abcd[4 * i + 3], type[i], order[i],
                       k[i] * KCALTOIU, phi0_deg[i] * PI / 180., mult[i]});
}
void orc_set_dihedrals(void* h, int nd, const int* abcd, const int* type, const int* order, const double* k,
                       const double* phi0_deg, const double* mult) {
    set_torsions(((Oracle*)h)->dihes, nd, abcd, type, order, k, phi0_deg, mult);
}
void orc_set_impropers(void* h, int nd, const int* abcd, const int* type, const int* order, const double* k,
                       const double* phi0_deg, const double* mult) {
    set_torsions(((Oracle*)h)->imprs, nd, abcd, type, order, k, phi0_deg, mult);
}

void orc_build_lists(void* h) { ((Oracle*)h)->build_lists(); }
void orc_update_verlet(void* h) { ((Oracle*)h)->update_verlet_list(); }

double orc_energy(void* h, double* ener10) {
    Oracle* o = (Oracle*)h;
    double e = o->getE();
    if (ener10) {
        double v[10] = {o->tot, o->pot, o->kin, o->elec, o->vdw, o->bond, o->ang, o->ub, o->dihe, o->impr};
        memcpy(ener10, v, sizeof v);
    }
    return e;
}

// Row accessors: return the row length; copy at most cap entries.
int orc_excl_row(void* h, int i, int* out, int cap) {
    Oracle* o = (Oracle*)h;
    int c = o->exclPair[i];
    for (int k = 0; k < c && k < cap; k++) out[k] = o->exclList[i][k];
    return c;
}
int orc_pairs14(void* h, int* out, int cap) {
    Oracle* o = (Oracle*)h;
    for (int k = 0; k < 2 * o->nPair14 && k < cap; k++) out[k] = o->neighList14[k];
    return o->nPair14;
}
int orc_verlet_row(void* h, int i, int* out, int cap) {
    Oracle* o = (Oracle*)h;
    if (o->neighPair.empty()) return 0;
    int c = o->neighPair[i];
    for (int k = 0; k < c && k < cap; k++) out[k] = o->neighList[i][k];
    return c;
}
long long orc_verlet_total(void* h) {
    Oracle* o = (Oracle*)h;
    long long t = 0;
    for (int c : o->neighPair) t += c;
    return t;
}

// Count of half-list pairs inside the cutoff (the unit of work "pair interaction").
long long orc_pairs_in_cutoff(void* h) {
    Oracle* o = (Oracle*)h;
    const double c2 = o->cutoff * o->cutoff;
    long long t = 0;
    double di[3], dj[3];
    for (int i = 0; i < o->n; i++) {
        if (o->neighPair.empty()) break;
        o->crd(i, di);
        for (int j : o->neighList[i]) { o->crd(j, dj); if (distance2(di, dj, o->pbc) <= c2) t++; }
    }
    return t;
}

// type: 1 TRN, 2 ROT; mode: 0 RESIDUE, 1 ALL, 2 ATOM; sele: natom flags.
int orc_add_move(void* h, int type, int mode, const int* sele, double dmax, double target, int each) {
    return ((Oracle*)h)->add_move(type, mode, sele, dmax, target, each);
}

int orc_move_instances(void* h, int t) { return (int)((Oracle*)h)->moves[t].inst.size(); }
// copies instance ranges as (first,last) pairs; returns the number of ranges
int orc_move_instance(void* h, int t, int k, int* ranges, int cap, int* pivot) {
    Oracle* o = (Oracle*)h;
    const std::vector<int>& l = o->moves[t].inst[k];
    int nr = 0;
    Oracle::for_ranges(l, [&](int a, int b) { if (2 * nr + 1 < cap) { ranges[2 * nr] = a; ranges[2 * nr + 1] = b; } nr++; });
    if (pivot) *pivot = o->moves[t].type == MV_ROT ? o->moves[t].pivot[k] : -2;
    return nr;
}

void orc_set_acceptance_units(void* h, int units) { ((Oracle*)h)->acceptance_units = units; }

int orc_mc_run(void* h, int nsteps, unsigned long long seed, double* trace, double* final_etot, long long* n_acc) {
    return ((Oracle*)h)->mc_run(nsteps, seed, trace, final_etot, n_acc);
}

// Local FP64 energy change of moving atoms idx[0..m) to (nx,ny,nz), over the current half
// Verlet list (switch mode) or all pairs (full mode), with the same cutoff, switch and exclusion
// rules as getE().  Equal to getE(after) - getE(before) up to the cancellation error of the
// difference of totals; used to check the device ΔE kernels.  Nonbonded only (no bonded terms).
double orc_delta_e(void* h, int m, const int* idx, const double* nx, const double* ny, const double* nz) {
    Oracle* o = (Oracle*)h;
    std::vector<double> ox(m), oy(m), oz(m);
    for (int k = 0; k < m; k++) { ox[k] = o->x[idx[k]]; oy[k] = o->y[idx[k]]; oz[k] = o->z[idx[k]]; }
    auto pairE = [&](int i, int j, bool fourteen) -> double {
        double di[3], dj[3];
        o->crd(i, di); o->crd(j, dj);
        double r2 = distance2(di, dj, o->pbc);
        const double ei = fourteen ? o->eps14[i] : o->eps[i], ej = fourteen ? o->eps14[j] : o->eps[j];
        const double si = fourteen ? o->sig14[i] : o->sig[i], sj = fourteen ? o->sig14[j] : o->sig[j];
        double rt = 1. / sqrt(r2);
        double pe = Oracle::eelec(o->q[i], o->q[j], rt), pv = Oracle::evdw(ei, ej, si, sj, rt);
        if (o->cutMode == CUT_SWITCH) {
            const double c2 = o->cutoff * o->cutoff, n2 = o->cuton * o->cuton;
            if (r2 > c2) return 0.0;
            if (r2 > n2) { double s1 = c2 - r2; double sw = X2<double>(s1) * (c2 + 2. * r2 - 3. * n2) * (1. / X3<double>(c2 - n2)); pe *= sw; pv *= sw; }
        }
        return CHGCHARMM * KCALTOIU * pe + 4.0 * pv;
    };
    // Pair set touching the moved atoms, each pair once.
    std::vector<char> moved(o->n, 0);
    for (int k = 0; k < m; k++) moved[idx[k]] = 1;
    std::vector<std::pair<int, int>> pairs;
    if (o->cutMode == CUT_SWITCH) {
        for (int i = 0; i < o->n; i++)
            for (int j : o->neighList[i]) if (moved[i] || moved[j]) pairs.push_back({i, j});
    } else {
        for (int i = 0; i < o->n - 1; i++) {
            int k = 0;
            for (int j = i + 1; j < o->n; j++) {
                bool ex = false;
                if (o->exclPair[i] > 0 && o->exclList[i][k] == j) { ex = true; k++; if (k >= o->exclPair[i]) k = o->exclPair[i] - 1; }
                if (!ex && (moved[i] || moved[j])) pairs.push_back({i, j});
            }
        }
    }
    std::vector<std::pair<int, int>> p14;
    for (int k = 0; k < o->nPair14; k++) {
        int i = o->neighList14[2 * k], j = o->neighList14[2 * k + 1];
        if (moved[i] || moved[j]) p14.push_back({i, j});
    }
    double eold = 0.0, enew = 0.0;
    for (auto& p : pairs) eold += pairE(p.first, p.second, false);
    for (auto& p : p14) eold += pairE(p.first, p.second, true);
    for (int k = 0; k < m; k++) { o->x[idx[k]] = nx[k]; o->y[idx[k]] = ny[k]; o->z[idx[k]] = nz[k]; }
    for (auto& p : pairs) enew += pairE(p.first, p.second, false);
    for (auto& p : p14) enew += pairE(p.first, p.second, true);
    for (int k = 0; k < m; k++) { o->x[idx[k]] = ox[k]; o->y[idx[k]] = oy[k]; o->z[idx[k]] = oz[k]; }
    return enew - eold;
}

}  // extern "C"
