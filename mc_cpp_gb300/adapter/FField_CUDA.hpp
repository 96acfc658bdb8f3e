// FField_CUDA: mc_cpp's FField interface (include/FField.hpp:52-153) backed by the GB300 engine.
//
// A drop-in for FField_MDBAS / FField_MDBAS_VECT: same constructor arguments, same getE()
// contract (total energy in internal units; in switch mode over the current Verlet list), same
// getE(double ener[10]) layout [tot, pot, kin = 0, elec, vdw, bond, ang, ub, dihe, impr] and the
// same askListUpdate(step).  Compiled as part of an mc_cpp build (it includes mc_cpp's headers)
// and linked against libmcgpu.so.
//
// Like every FField it holds references to the caller's AtomList, PerConditions and Ensemble and
// reads the coordinates again on every getE(), because MC_metropolis moves atoms in place between
// calls (Move.hpp:47-48, AtomList.cpp:427).  getE() hands the AtomList's coordinate vectors to
// mcg_energy_host, which sends the device only what changed since the previous call: nothing
// before a move (or after a rejected one), a commit after an accepted one, the moved atoms' dE
// after a move.  So the unmodified MC_metropolis loop costs one small dE launch per trial move, not
// two full energies.  askListUpdate() first brings the device up to the AtomList, then rebuilds
// the list; the next getE() recomputes the whole energy over the new list.  getE() refreshes the
// tot and pot members; getE(double ener[10]) recomputes every component.  The device system is
// created on the first energy call, after IO_MDBAS has filled the bonded lists through the
// setters; its exclusion and Verlet lists are built on the device with the same rules as
// List_nonBonded.
//
// Errors follow the reference's convention: the reason goes to cerr and the process exits with
// the engine's negative status (FField_MDBAS.cpp:68-71 does the same for a bad cut mode).
#ifndef FFIELD_CUDA_H
#define FFIELD_CUDA_H

#include <string>
#include <vector>

#include "FField.hpp"
#include "mcg.h"

class FField_CUDA : public FField
{
public:
    // precision: MCG_PREC_FP64 (plain, the reference's arithmetic) or MCG_PREC_MIXED
    FField_CUDA(AtomList& _at_List, PerConditions& _pbc, Ensemble& _ens, std::string _cutMode = "switch",
                double _ctoff = 12.0, double _cuton = 10.0, double _dcut = 2.0, int precision = MCG_PREC_FP64);
    virtual ~FField_CUDA();

    virtual double getE();
    virtual void getE(double ener[10]);
    virtual void askListUpdate(int st);

    // Energy change (internal units) of moving atoms[0..n) to (x, y, z), against the current
    // coordinates and Verlet list: what MC_metropolis obtains as getE() after the move minus
    // getE() before it, without touching the AtomList and without recomputing the whole system.
    double getDeltaE(int n, const int* atoms, const double* x, const double* y, const double* z);

protected:
    virtual double getEtot();
    virtual double getEswitch();
    virtual void computeNonBonded_full();
    virtual void computeNonBonded14();
    virtual void computeNonBonded_switch();
    virtual void computeNonBonded14_switch();
    virtual void computeEbond();
    virtual void computeEang();
    virtual void computeEub();
    virtual void computeEdihe();
    virtual void computeEimpr();

private:
    mcg_system* sys;
    int precision;
    std::vector<double> cx, cy, cz;

    void ensure();                  // device system on first use
    void upload();                  // AtomList coordinates -> device
    void compute();                 // all components into the FField members
    static void check(int rc, const char* what);
};

#endif // FFIELD_CUDA_H
