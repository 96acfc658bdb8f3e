// MDBAS input files on the host: the .cor coordinate file and the forcefield file, read as the
// reference's IO_MDBAS does (src/IO_MDBAS.cpp:77-128 read_coord, :130-505 read_ff), into arrays
// owned by the library.  Values stay in file units (kcal/mol, Angstrom, degrees, file epsilon);
// build_host_system converts them like read_ff when a system is created from them.
//
// .cor: title lines starting with '*', a line whose first token is the atom count, then ten
// whitespace-separated fields per atom (id, global residue id, residue name, atom name, x, y, z,
// segment, residue id in segment, weight).
// forcefield: keyword lines (case-insensitive) `atoms N`, `bonds N`, `constraints N`,
// `urey-bradley N`, `angles N`, `dihedrals N`, `impropers N`, `vdw N`, `end`, each followed by N
// records; lines starting with '#' are comments.  Atom indices in the file are 1-based.
#include <algorithm>
#include <cctype>
#include <cmath>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "engine.hpp"
#include "mcg.h"

struct mcg_mdbas {
    int natom = 0;
    std::vector<double> x, y, z, q, mass, eps, sig, eps14, sig14;
    std::vector<unsigned char> frozen;
    std::vector<int> resid;
    std::vector<int> bond_atoms, bond_type, ub_atoms, angle_atoms, angle_type, dihe_atoms, dihe_type, dihe_order,
        impr_atoms, impr_type, impr_order;
    std::vector<double> bond_k, bond_r0, bond_beta, ub_k, ub_r0, angle_k, angle_theta0, dihe_k, dihe_phi0, dihe_mult,
        impr_k, impr_phi0, impr_mult;
};

namespace {

using mcg::fail;

std::vector<std::string> tokens(const std::string& line) {
    std::istringstream is(line);
    std::vector<std::string> t;
    std::string w;
    while (is >> w) t.push_back(w);
    return t;
}

bool to_int(const std::string& s, int& v) {
    char* end = nullptr;
    const long r = std::strtol(s.c_str(), &end, 10);
    if (end == s.c_str() || *end) return false;
    v = (int)r;
    return true;
}

bool to_double(const std::string& s, double& v) {
    char* end = nullptr;
    v = std::strtod(s.c_str(), &end);
    return end != s.c_str() && !*end;
}

int read_cor(const char* path, mcg_mdbas& m) {
    std::ifstream f(path);
    if (!f) return fail(MCG_EIO, std::string("cannot open coordinate file ") + path);
    std::string line;
    while (std::getline(f, line) && !line.empty() && line[0] == '*') {}
    std::vector<std::string> head = tokens(line);
    int n = 0;
    if (head.empty() || !to_int(head[0], n) || n <= 0) return fail(MCG_EIO, std::string("no atom count in ") + path);
    std::vector<std::string> all;
    while (std::getline(f, line)) {
        std::vector<std::string> t = tokens(line);
        all.insert(all.end(), t.begin(), t.end());
    }
    if ((int64_t)all.size() < 10 * (int64_t)n) return fail(MCG_EIO, std::string("truncated coordinate file ") + path);
    m.natom = n;
    m.x.resize(n); m.y.resize(n); m.z.resize(n); m.resid.resize(n);
    for (int i = 0; i < n; i++) {
        const std::string* r = &all[10 * (size_t)i];
        if (!to_int(r[1], m.resid[i]) || !to_double(r[4], m.x[i]) || !to_double(r[5], m.y[i]) || !to_double(r[6], m.z[i]))
            return fail(MCG_EIO, "bad coordinate record for atom " + std::to_string(i + 1));
    }
    return MCG_OK;
}

struct FFReader {
    std::ifstream f;
    int lineno = 0;
    // next non-comment record of at least `need` tokens
    int record(size_t need, std::vector<std::string>& t) {
        std::string line;
        while (std::getline(f, line)) {
            lineno++;
            if (!line.empty() && line[0] == '#') continue;
            t = tokens(line);
            if (t.size() < need) return fail(MCG_EIO, "forcefield line " + std::to_string(lineno) + ": too few fields");
            return MCG_OK;
        }
        return fail(MCG_EIO, "truncated forcefield file");
    }
};

int read_ff(const char* path, mcg_mdbas& m) {
    FFReader R;
    R.f.open(path);
    if (!R.f) return fail(MCG_EIO, std::string("cannot open forcefield file ") + path);
    const int n = m.natom;
    m.q.assign(n, 0.0); m.mass.assign(n, 0.0); m.frozen.assign(n, 0);
    m.eps.assign(n, 0.0); m.sig.assign(n, 0.0); m.eps14.assign(n, 0.0); m.sig14.assign(n, 0.0);
    std::string line;
    std::vector<std::string> t;
    auto atom = [&](const std::string& s, int& a) {
        if (!to_int(s, a) || a < 1 || a > n) return false;
        a -= 1;
        return true;
    };
    auto bad = [&](const char* what) { return fail(MCG_EIO, std::string("forcefield: bad ") + what + " record near line " + std::to_string(R.lineno)); };
    while (std::getline(R.f, line)) {
        R.lineno++;
        if (!line.empty() && line[0] == '#') continue;
        std::vector<std::string> head = tokens(line);
        if (head.empty()) continue;
        std::string key = head[0];
        std::transform(key.begin(), key.end(), key.begin(), [](unsigned char c) { return (char)std::tolower(c); });
        if (key == "end") break;
        int cnt = 0;
        if (head.size() < 2 || !to_int(head[1], cnt) || cnt < 0) return fail(MCG_EIO, "forcefield: keyword '" + key + "' without a count");
        if (key == "atoms") {
            if (cnt != n) return fail(MCG_EIO, "forcefield atom count differs from the coordinate file");
            for (int k = 0; k < cnt; k++) {
                int a, ty, fr;
                if (R.record(6, t) || !atom(t[0], a) || !to_int(t[2], ty) || !to_double(t[3], m.q[a]) ||
                    !to_double(t[4], m.mass[a]) || !to_int(t[5], fr))
                    return bad("atoms");
                m.frozen[a] = fr ? 1 : 0;
            }
        } else if (key == "bonds") {
            for (int k = 0; k < cnt; k++) {
                int a, b, ty;
                double kk, r0, be;
                if (R.record(6, t) || !atom(t[0], a) || !atom(t[1], b) || !to_int(t[2], ty) || !to_double(t[3], kk) ||
                    !to_double(t[4], r0) || !to_double(t[5], be))
                    return bad("bonds");
                m.bond_atoms.push_back(a); m.bond_atoms.push_back(b); m.bond_type.push_back(ty);
                m.bond_k.push_back(kk); m.bond_r0.push_back(r0); m.bond_beta.push_back(be);
            }
        } else if (key == "constraints") {
            // the reference never leaves a non-empty constraints section (IO_MDBAS.cpp:236-262)
            if (cnt) return fail(MCG_ENOTSUP, "forcefield: constraints are not supported");
        } else if (key == "urey-bradley") {
            for (int k = 0; k < cnt; k++) {
                int a, b;
                double kk, r0;
                if (R.record(4, t) || !atom(t[0], a) || !atom(t[1], b) || !to_double(t[2], kk) || !to_double(t[3], r0))
                    return bad("urey-bradley");
                m.ub_atoms.push_back(a); m.ub_atoms.push_back(b); m.ub_k.push_back(kk); m.ub_r0.push_back(r0);
            }
        } else if (key == "angles") {
            for (int k = 0; k < cnt; k++) {
                int a, b, c, ty;
                double kk, th;
                if (R.record(6, t) || !atom(t[0], a) || !atom(t[1], b) || !atom(t[2], c) || !to_int(t[3], ty) ||
                    !to_double(t[4], kk) || !to_double(t[5], th))
                    return bad("angles");
                m.angle_atoms.insert(m.angle_atoms.end(), {a, b, c});
                m.angle_type.push_back(ty); m.angle_k.push_back(kk); m.angle_theta0.push_back(th);
            }
        } else if (key == "dihedrals" || key == "impropers") {
            const bool dih = key == "dihedrals";
            for (int k = 0; k < cnt; k++) {
                int a, b, c, d, ty, od;
                double kk, ph, mu;
                if (R.record(9, t) || !atom(t[0], a) || !atom(t[1], b) || !atom(t[2], c) || !atom(t[3], d) ||
                    !to_int(t[4], ty) || !to_int(t[5], od) || !to_double(t[6], kk) || !to_double(t[7], ph) || !to_double(t[8], mu))
                    return bad(dih ? "dihedrals" : "impropers");
                (dih ? m.dihe_atoms : m.impr_atoms).insert((dih ? m.dihe_atoms : m.impr_atoms).end(), {a, b, c, d});
                (dih ? m.dihe_type : m.impr_type).push_back(ty);
                (dih ? m.dihe_order : m.impr_order).push_back(od);
                (dih ? m.dihe_k : m.impr_k).push_back(kk);
                (dih ? m.dihe_phi0 : m.impr_phi0).push_back(ph);
                (dih ? m.dihe_mult : m.impr_mult).push_back(mu);
            }
        } else if (key == "vdw") {
            if (cnt != n) return fail(MCG_EIO, "forcefield vdw count differs from the atom count");
            for (int k = 0; k < cnt; k++) {
                int a;
                if (R.record(7, t) || !atom(t[0], a)) return bad("vdw");
                // IO_MDBAS.cpp:452-456: records must come in atom order
                if (a != k) return fail(MCG_EIO, "forcefield: vdw parameters missing for atom " + std::to_string(k + 1));
                if (!to_double(t[2], m.eps[a]) || !to_double(t[3], m.sig[a]) || !to_double(t[5], m.eps14[a]) ||
                    !to_double(t[6], m.sig14[a]))
                    return bad("vdw");
            }
        } else {
            return fail(MCG_EIO, "forcefield: unknown keyword '" + key + "'");
        }
    }
    return MCG_OK;
}

}  // namespace

extern "C" {

int mcg_mdbas_read(const char* cor_path, const char* ff_path, mcg_mdbas** out) {
    if (!out) return fail(MCG_EINVAL, "null output");
    *out = nullptr;
    if (!cor_path || !ff_path) return fail(MCG_EINVAL, "null path");
    mcg_mdbas* m = new mcg_mdbas;
    int r = read_cor(cor_path, *m);
    if (!r) r = read_ff(ff_path, *m);
    if (r) { delete m; return r; }
    *out = m;
    return MCG_OK;
}

int mcg_mdbas_natom(const mcg_mdbas* m) { return m ? m->natom : 0; }

int mcg_mdbas_fill(const mcg_mdbas* m, mcg_system_desc* d) {
    if (!m || !d) return fail(MCG_EINVAL, "null argument");
    d->natom = m->natom;
    d->x = m->x.data(); d->y = m->y.data(); d->z = m->z.data(); d->q = m->q.data();
    d->eps = m->eps.data(); d->sig = m->sig.data(); d->eps14 = m->eps14.data(); d->sig14 = m->sig14.data();
    d->mass = m->mass.data(); d->frozen = m->frozen.data(); d->resid = m->resid.data();
    d->nbond = (int)m->bond_type.size();
    d->bond_atoms = m->bond_atoms.data(); d->bond_type = m->bond_type.data();
    d->bond_k = m->bond_k.data(); d->bond_r0 = m->bond_r0.data(); d->bond_beta = m->bond_beta.data();
    d->nub = (int)m->ub_k.size();
    d->ub_atoms = m->ub_atoms.data(); d->ub_k = m->ub_k.data(); d->ub_r0 = m->ub_r0.data();
    d->nangle = (int)m->angle_type.size();
    d->angle_atoms = m->angle_atoms.data(); d->angle_type = m->angle_type.data();
    d->angle_k = m->angle_k.data(); d->angle_theta0 = m->angle_theta0.data();
    d->ndihe = (int)m->dihe_type.size();
    d->dihe_atoms = m->dihe_atoms.data(); d->dihe_type = m->dihe_type.data(); d->dihe_order = m->dihe_order.data();
    d->dihe_k = m->dihe_k.data(); d->dihe_phi0 = m->dihe_phi0.data(); d->dihe_mult = m->dihe_mult.data();
    d->nimpr = (int)m->impr_type.size();
    d->impr_atoms = m->impr_atoms.data(); d->impr_type = m->impr_type.data(); d->impr_order = m->impr_order.data();
    d->impr_k = m->impr_k.data(); d->impr_phi0 = m->impr_phi0.data(); d->impr_mult = m->impr_mult.data();
    d->param_units = MCG_UNITS_FILE;
    return MCG_OK;
}

int mcg_mdbas_free(mcg_mdbas* m) {
    delete m;
    return MCG_OK;
}

}  // extern "C"
