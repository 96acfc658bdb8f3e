// Internal declarations shared by the host runtime (.cpp) and the sm_103a kernels (.cu).
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include "mcg.h"

namespace mcg {

// Constants of the reference, include/Constants.hpp:24-45.
constexpr double KCALTOIU = 418.4;
constexpr double CHGCHARMM = 332.0716;
constexpr double RBOLTZUI = 0.83144621;
constexpr double PI = 3.141592653589793;
constexpr double TWOPI = 6.283185307179586;

// Thread-local error text for mcg_last_error().
void set_error(const std::string& msg);
int fail(int code, const std::string& msg);

struct BondT { int a, b, type; double k, r0, beta; };
struct AngleT { int a, b, c, type; double k, theta0; };
struct TorsT { int a, b, c, d, type, order; double k, phi0, mult; };

// Host-side system model: AtomList + PerConditions + FField settings + topology, with the
// reference's unit conversions applied (epsilon stored as sqrt(eps*418.4), k*418.4, radians).
struct HostSystem {
    int n = 0;
    int pbc = MCG_PBC_NONE;
    double L[3] = {0, 0, 0}, rL[3] = {0, 0, 0};
    int cut = MCG_CUT_SWITCH;
    double rc = 12, ron = 10, dcut = 2, temp = 300;
    int prec = MCG_PREC_FP64;
    std::vector<double> x, y, z, q, eps, sig, eps14, sig14, mass;
    std::vector<uint8_t> frozen;
    std::vector<int> resid;
    std::vector<BondT> bonds, ubs;
    std::vector<AngleT> angles;
    std::vector<TorsT> dihes, imprs;
    // Exclusion rows exactly as List_nonBonded stores them (first exclPair[i] entries of
    // exclList[i], after the wrap rotation): CSR.
    std::vector<int> exclStart, exclCount, exclData;
    // Full-mode effective rows: the entries computeNonBonded_full's cursor can match
    // (FField_MDBAS.cpp:227-234): the strictly increasing run of stored entries above i.
    std::vector<int> fexclStart, fexclCount, fexclData;
    std::vector<int> pairs14;  // 2 * n14, (i, j) in the reference's order
    int maxExclSpan = 0;       // max over rows of (entry - i) for entries above i
};

// Builds a HostSystem from the ABI description (validates, converts units, builds exclusions).
int build_host_system(const mcg_system_desc* d, HostSystem& hs);

// List_nonBonded::build_exclude_list (List_nonBonded.cpp:143-775) on the host.
void build_exclusions(HostSystem& hs);

// One registered move type (List_Moves restated, List_Moves.cpp:257-457).
struct MoveKind {
    int type = MCG_MOVE_TRN, mode = MCG_MODE_RESIDUE;
    double dmax = 0.5, target = 50.0;
    int each = 0;
    // instance k covers ranges[rstart[k] .. rstart[k+1]) of (first,last) atom pairs
    std::vector<int> rstart, ranges, pivot;
    int ninst() const { return (int)rstart.size() - 1; }
};
int build_move_kind(const HostSystem& hs, int type, int mode, const int* sele, double dmax, double target,
                    int each, MoveKind& out);

}  // namespace mcg
