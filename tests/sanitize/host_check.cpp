// Host code under AddressSanitizer + UndefinedBehaviorSanitizer.  Linked with the library's
// host-only sources (mc_cpp_gb300/csrc/mdbas_io.cpp, topology.cpp) and the oracle
// (oracle/mc_oracle.cpp), all built with -fsanitize=address,undefined by tests/test_sanitizers.py.
//
// usage: host_check SYSTEM.cor SYSTEM.ff SETTINGS MOVES [BAD.cor BAD.ff]...
//   SETTINGS: one line "pbc a b c cut cutoff cuton dcut temp"
//   MOVES:    one line per move type "type mode resid_lo resid_hi dmax target each" (atoms whose
//             residue id lies in [resid_lo, resid_hi] are selected)
// It reads the system through the MDBAS reader, builds the host system (unit conversion,
// exclusion and 1-4 lists) and every move type's instances, then drives the oracle through
// lists, energies, one dE and a short Metropolis run; every bad file pair must be rejected with an
// error status.  Prints "key value" lines that the test compares with the unsanitized builds.
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "engine.hpp"
#include "mcg.h"

namespace mcg {
const char* last_error_cstr();
}

extern "C" {
void* orc_create(int natom, int pbc_type, double a, double b, double c, int cut_mode, double cutoff, double cuton,
                 double deltacut, double temp);
void orc_destroy(void* h);
void orc_set_atoms(void* h, const double* x, const double* y, const double* z, const double* q, const double* eps_file,
                   const double* sig, const double* eps14_file, const double* sig14, const double* mass,
                   const unsigned char* frozen, const int* resid);
void orc_set_bonds(void* h, int nb, const int* ab, const int* type, const double* k, const double* r0, const double* beta);
void orc_set_ub(void* h, int nb, const int* ab, const double* k, const double* r0);
void orc_set_angles(void* h, int na, const int* abc, const int* type, const double* k, const double* theta0_deg);
void orc_set_dihedrals(void* h, int nd, const int* abcd, const int* type, const int* order, const double* k,
                       const double* phi0_deg, const double* mult);
void orc_set_impropers(void* h, int nd, const int* abcd, const int* type, const int* order, const double* k,
                       const double* phi0_deg, const double* mult);
void orc_build_lists(void* h);
double orc_energy(void* h, double* ener10);
long long orc_verlet_total(void* h);
int orc_add_move(void* h, int type, int mode, const int* sele, double dmax, double target, int each);
int orc_mc_run(void* h, int nsteps, unsigned long long seed, double* trace, double* final_etot, long long* n_acc);
double orc_delta_e(void* h, int m, const int* idx, const double* nx, const double* ny, const double* nz);
}

struct Move {
    int type, mode, lo, hi, each;
    double dmax, target;
};

int main(int argc, char** argv) {
    if (argc < 5 || (argc - 5) % 2 != 0) {
        std::fprintf(stderr, "usage: host_check cor ff settings moves [bad.cor bad.ff]...\n");
        return 2;
    }
    mcg_system_desc d = {};
    {
        FILE* f = std::fopen(argv[3], "r");
        if (!f || std::fscanf(f, "%d %lf %lf %lf %d %lf %lf %lf %lf", &d.pbc_type, &d.box[0], &d.box[1], &d.box[2],
                              &d.cut_mode, &d.cutoff, &d.cuton, &d.dcut, &d.temp) != 9) {
            std::fprintf(stderr, "bad settings file\n");
            return 2;
        }
        std::fclose(f);
    }
    std::vector<Move> moves;
    {
        FILE* f = std::fopen(argv[4], "r");
        if (!f) return 2;
        Move m;
        while (std::fscanf(f, "%d %d %d %d %lf %lf %d", &m.type, &m.mode, &m.lo, &m.hi, &m.dmax, &m.target, &m.each) == 7)
            moves.push_back(m);
        std::fclose(f);
    }

    // the library's reader, host system and move builders
    mcg_mdbas* md = nullptr;
    if (mcg_mdbas_read(argv[1], argv[2], &md) != MCG_OK) {
        std::fprintf(stderr, "read failed: %s\n", mcg::last_error_cstr());
        return 3;
    }
    if (mcg_mdbas_fill(md, &d) != MCG_OK) return 3;
    mcg::HostSystem hs;
    if (mcg::build_host_system(&d, hs) != MCG_OK) {
        std::fprintf(stderr, "host system: %s\n", mcg::last_error_cstr());
        return 4;
    }
    const int n = d.natom;
    std::printf("natom %d\n", n);
    std::printf("excl_total %zu\n", hs.exclData.size());
    std::printf("pairs14 %zu\n", hs.pairs14.size() / 2);
    std::vector<std::vector<int>> seles;
    for (size_t t = 0; t < moves.size(); t++) {
        std::vector<int> sele(n, 0);
        for (int i = 0; i < n; i++) sele[i] = (d.resid[i] >= moves[t].lo && d.resid[i] <= moves[t].hi) ? 1 : 0;
        mcg::MoveKind mk;
        if (mcg::build_move_kind(hs, moves[t].type, moves[t].mode, sele.data(), moves[t].dmax, moves[t].target,
                                 moves[t].each, mk) != MCG_OK) {
            std::fprintf(stderr, "move kind %zu: %s\n", t, mcg::last_error_cstr());
            return 5;
        }
        std::printf("instances_%zu %d\n", t, mk.ninst());
        seles.push_back(sele);
    }

    // the oracle on the same description
    void* o = orc_create(n, d.pbc_type, d.box[0], d.box[1], d.box[2], d.cut_mode, d.cutoff, d.cuton, d.dcut, d.temp);
    orc_set_atoms(o, d.x, d.y, d.z, d.q, d.eps, d.sig, d.eps14, d.sig14, d.mass, d.frozen, d.resid);
    if (d.nbond) orc_set_bonds(o, d.nbond, d.bond_atoms, d.bond_type, d.bond_k, d.bond_r0, d.bond_beta);
    if (d.nub) orc_set_ub(o, d.nub, d.ub_atoms, d.ub_k, d.ub_r0);
    if (d.nangle) orc_set_angles(o, d.nangle, d.angle_atoms, d.angle_type, d.angle_k, d.angle_theta0);
    if (d.ndihe) orc_set_dihedrals(o, d.ndihe, d.dihe_atoms, d.dihe_type, d.dihe_order, d.dihe_k, d.dihe_phi0, d.dihe_mult);
    if (d.nimpr) orc_set_impropers(o, d.nimpr, d.impr_atoms, d.impr_type, d.impr_order, d.impr_k, d.impr_phi0, d.impr_mult);
    orc_build_lists(o);
    for (size_t t = 0; t < moves.size(); t++)
        if (orc_add_move(o, moves[t].type, moves[t].mode, seles[t].data(), moves[t].dmax, moves[t].target, moves[t].each) < 0)
            return 6;
    double e10[10];
    orc_energy(o, e10);
    std::printf("energy %.17g\n", e10[0]);
    std::printf("verlet_total %lld\n", orc_verlet_total(o));
    {
        // dE of the second residue shifted by (0.1, -0.05, 0.07)
        std::vector<int> idx;
        std::vector<double> nx, ny, nz;
        for (int i = 0; i < n; i++)
            if (d.resid[i] == 2) {
                idx.push_back(i);
                nx.push_back(d.x[i] + 0.1);
                ny.push_back(d.y[i] - 0.05);
                nz.push_back(d.z[i] + 0.07);
            }
        std::printf("delta_e %.17g\n", orc_delta_e(o, (int)idx.size(), idx.data(), nx.data(), ny.data(), nz.data()));
    }
    double fe = 0.0;
    long long nacc = 0;
    if (orc_mc_run(o, 120, 1234ULL, nullptr, &fe, &nacc) != 0) return 7;
    std::printf("mc_final %.17g\n", fe);
    std::printf("mc_accepted %lld\n", nacc);
    orc_destroy(o);
    mcg_mdbas_free(md);

    // malformed inputs: rejected with a status, never read out of bounds
    for (int a = 5; a + 1 < argc; a += 2) {
        mcg_mdbas* bad = nullptr;
        const int rc = mcg_mdbas_read(argv[a], argv[a + 1], &bad);
        std::printf("bad_%d %d\n", (a - 5) / 2, rc);
        if (rc == MCG_OK) mcg_mdbas_free(bad);
    }
    return 0;
}
