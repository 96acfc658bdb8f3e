// ref_math.hpp — the reference's FP64 pair geometry and constants, shared by the oracle
// restatements (mc_oracle.cpp, batch_oracle.cpp).  TEST INFRASTRUCTURE ONLY (see mc_oracle.cpp).
// Included inside each file's anonymous namespace.
#pragma once

constexpr double KCALTOIU = 418.4;          // Constants.hpp:29
constexpr double CHGCHARMM = 332.0716;      // Constants.hpp:36
constexpr double RBOLTZUI = 0.83144621;     // Constants.hpp:34
constexpr double PI = 3.141592653589793;    // Constants.hpp:40
constexpr double TWOPI = 6.283185307179586; // Constants.hpp:41

enum { PBC_NONE = 0, PBC_CUBIC = 1, PBC_ORBIC = 2 };

// Tools::rint, Tools.hpp:221-224: round half away from zero through an int cast.
inline double ref_rint(double x) { return (double)(x >= 0. ? (int)(x + 0.5) : (int)(x - 0.5)); }

struct Pbc {
    int type = PBC_NONE;
    double L[3] = {0, 0, 0}, rL[3] = {0, 0, 0};
    // PerConditions::applyPBC(double[3]), PerConditions.cpp:244-285
    inline void apply(double d[3]) const {
        if (type == PBC_CUBIC || type == PBC_ORBIC) {
            d[0] -= L[0] * ref_rint(rL[0] * d[0]);
            d[1] -= L[1] * ref_rint(rL[1] * d[1]);
            d[2] -= L[2] * ref_rint(rL[2] * d[2]);
        }
    }
};

// Tools::distance2, Tools.hpp:151-188: delta = a2 - a1, MIC, r^2.
inline double distance2(const double a1[3], const double a2[3], const Pbc& pbc, double d[3]) {
    d[0] = a2[0] - a1[0];
    d[1] = a2[1] - a1[1];
    d[2] = a2[2] - a1[2];
    pbc.apply(d);
    return d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
}
inline double distance2(const double a1[3], const double a2[3], const Pbc& pbc) {
    double d[3];
    return distance2(a1, a2, pbc, d);
}
template <typename T> inline T X2(T x) { return x * x; }
template <typename T> inline T X3(T x) { return x * x * x; }
template <typename T> inline T X6(T x) { return x * x * x * x * x * x; }
template <typename T> inline T X12(T x) { return x * x * x * x * x * x * x * x * x * x * x * x; }
