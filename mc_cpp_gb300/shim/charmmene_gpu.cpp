// libcharmmene_gpu.so: the reference's Fortran/C energy interface (src/FORTRAN_interface.cpp:23-106)
// on top of libmcgpu.so's C ABI.  Same seven symbols, same arguments, same units (kcal/mol out),
// same one-system-per-process state.  Errors print to stderr and exit with the library's negative
// status, the reference's convention for bad input.
#include <cctype>
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include "charmmene_gpu.h"
#include "mcg.h"

namespace {

struct State {
    int pbc = MCG_PBC_NONE;
    double box[3] = {0, 0, 0};
    int natom = 0;
    double temp = 0;
    mcg_mdbas* files = nullptr;
    mcg_system* sys = nullptr;
    std::vector<double> x, y, z;
};
State g;

std::string clean(const char* s) {
    // Tools::str_rm_blank_spaces + str_to_lower_case (Tools.hpp)
    std::string out;
    for (const char* p = s; p && *p; p++)
        if (!std::isspace((unsigned char)*p)) out.push_back((char)std::tolower((unsigned char)*p));
    return out;
}

std::string strip(const char* s) {
    std::string out;
    for (const char* p = s; p && *p; p++)
        if (!std::isspace((unsigned char)*p)) out.push_back(*p);
    return out;
}

void die(int rc, const char* what) {
    std::fprintf(stderr, "Error : %s: %s\n", what, mcg_last_error());
    std::exit(rc < 0 ? rc : -1);
}

void need_system(const char* fn) {
    if (!g.sys) {
        std::fprintf(stderr, "Error : %s called before set_ff_and_cor_\n", fn);
        std::exit(-1);
    }
}

}  // namespace

extern "C" {

void set_pbc_(char* type, double* a, double* b, double* c, double* alpha, double* beta, double* gamma) {
    const std::string t = clean(type);
    if (t == "none") g.pbc = MCG_PBC_NONE;
    else if (t == "cubic") g.pbc = MCG_PBC_CUBIC;
    else if (t == "orbic") g.pbc = MCG_PBC_ORBIC;
    else {
        std::fprintf(stderr, "Error : periodic boundary type '%s' is not supported\n", t.c_str());
        std::exit(-1);
    }
    (void)alpha; (void)beta; (void)gamma;   // orthogonal boxes only, as the reference's MIC
    g.box[0] = *a;
    g.box[1] = g.pbc == MCG_PBC_CUBIC ? *a : *b;
    g.box[2] = g.pbc == MCG_PBC_CUBIC ? *a : *c;
}

void set_ens_(int* natom, double* Temp) {
    g.natom = *natom;
    g.temp = *Temp;
}

void set_ff_and_cor_(char* cutoffmode, double* ctoff, double* cton, double* dcut, char* FF_file, char* COR_file) {
    const std::string mode = clean(cutoffmode);
    if (mode != "full" && mode != "switch") {
        std::fprintf(stderr, "Error : cut mode '%s' is not supported ('full' or 'switch')\n", mode.c_str());
        std::exit(-50);
    }
    if (g.sys) { mcg_destroy(g.sys); g.sys = nullptr; }
    if (g.files) { mcg_mdbas_free(g.files); g.files = nullptr; }
    int rc = mcg_mdbas_read(strip(COR_file).c_str(), strip(FF_file).c_str(), &g.files);
    if (rc) die(rc, "reading the MDBAS input");
    if (g.natom && mcg_mdbas_natom(g.files) != g.natom) {
        std::fprintf(stderr, "Error : set_ens_ gave %d atoms, the coordinate file holds %d\n", g.natom,
                     mcg_mdbas_natom(g.files));
        std::exit(-1);
    }
    mcg_system_desc d = {};
    mcg_mdbas_fill(g.files, &d);
    d.pbc_type = g.pbc;
    for (int k = 0; k < 3; k++) d.box[k] = g.box[k];
    d.cut_mode = mode == "switch" ? MCG_CUT_SWITCH : MCG_CUT_FULL;
    d.cutoff = *ctoff;
    d.cuton = *cton;
    d.dcut = *dcut;
    d.temp = g.temp;
    d.precision = MCG_PREC_FP64;
    rc = mcg_create(&d, &g.sys);
    if (rc) die(rc, "creating the device system");
    g.natom = d.natom;
    g.x.resize(g.natom); g.y.resize(g.natom); g.z.resize(g.natom);
}

void get_energy_(double ener[10]) {
    need_system("get_energy_");
    const int rc = mcg_energy(g.sys, ener);
    if (rc) die(rc, "energy");
    for (int i = 0; i < 10; i++) ener[i] /= 418.4;   // CONSTANTS::kcaltoiu
}

void set_coords_(double x[], double y[], double z[]) {
    need_system("set_coords_");
    const int rc = mcg_set_coords(g.sys, x, y, z);
    if (rc) die(rc, "set_coords_");
}

void get_mass_(double mass[]) {
    need_system("get_mass_");
    mcg_system_desc d = {};
    mcg_mdbas_fill(g.files, &d);
    for (int i = 0; i < g.natom; i++) mass[i] = d.mass[i];
}

void clean_(void) {
    if (g.sys) mcg_destroy(g.sys);
    if (g.files) mcg_mdbas_free(g.files);
    g = State();
}

}  // extern "C"
