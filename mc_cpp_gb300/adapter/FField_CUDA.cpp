// FField_CUDA: see FField_CUDA.hpp.  Marshals mc_cpp's objects into the engine's C ABI
// (include/mcg.h); no arithmetic of its own.
#include "FField_CUDA.hpp"

#include <chrono>
#include <cstdlib>
#include <iostream>

FField_CUDA::FField_CUDA(AtomList& _at_List, PerConditions& _pbc, Ensemble& _ens, std::string _cutMode,
                         double _ctoff, double _cuton, double _dcut, int _precision)
    : FField(_at_List, _pbc, _ens, _cutMode, _ctoff, _cuton, _dcut), sys(nullptr), precision(_precision)
{
}

FField_CUDA::~FField_CUDA()
{
    if (sys)
        mcg_destroy(sys);
}

void FField_CUDA::check(int rc, const char* what)
{
    if (rc != MCG_OK)
    {
        std::cerr << "Error : FField_CUDA " << what << " failed (status " << rc << ") : " << mcg_last_error() << std::endl;
        std::exit(rc);
    }
}

void FField_CUDA::ensure()
{
    if (sys)
        return;
    const int n = ens.getN();
    std::vector<double> q(n), eps(n), sig(n), eps14(n), sig14(n), mass(n);
    std::vector<unsigned char> frozen(n);
    std::vector<int> resid(n);
    cx.resize(n); cy.resize(n); cz.resize(n);
    const std::vector<bool>& fr = at_List.getFrozenList();
    for (int i = 0; i < n; i++)
    {
        cx[i] = at_List.getX(i); cy[i] = at_List.getY(i); cz[i] = at_List.getZ(i);
        q[i] = at_List.getCharge(i);
        eps[i] = at_List.getEpsilon(i);        // already sqrt(eps * kcaltoiu) (IO_MDBAS.cpp:460)
        sig[i] = at_List.getSigma(i);
        eps14[i] = at_List.getEpsilon14(i);
        sig14[i] = at_List.getSigma14(i);
        mass[i] = at_List.getMass(i);
        frozen[i] = (i < (int)fr.size() && fr[i]) ? 1 : 0;
        resid[i] = at_List.getResidue_id_global(i);
    }
    std::vector<int> ba, bt, ua, aa, at, da, dt, dord, ia, it, iord;
    std::vector<double> bk, br, bb, uk, ur, ak, ath, dk, dph, dm, ik, iph, im;
    for (const Bond& b : bndList)
    {
        ba.push_back(b.getAt1()); ba.push_back(b.getAt2()); bt.push_back(b.getType());
        bk.push_back(b.getK()); br.push_back(b.getR0()); bb.push_back(b.getBeta());
    }
    for (const Bond_UB& b : ubList)
    {
        ua.push_back(b.getAt1()); ua.push_back(b.getAt2()); uk.push_back(b.getK()); ur.push_back(b.getR0());
    }
    for (const Angle& a : angList)
    {
        aa.push_back(a.getAt1()); aa.push_back(a.getAt2()); aa.push_back(a.getAt3());
        at.push_back(a.getType()); ak.push_back(a.getK()); ath.push_back(a.getTheta0());
    }
    for (const Dihedral& d : diheList)
    {
        da.push_back(d.getAt1()); da.push_back(d.getAt2()); da.push_back(d.getAt3()); da.push_back(d.getAt4());
        dt.push_back(d.getType()); dord.push_back(d.getOrder());
        dk.push_back(d.getK()); dph.push_back(d.getPhi0()); dm.push_back(d.getMult());
    }
    for (const Dihedral_improper& d : imprList)
    {
        ia.push_back(d.getAt1()); ia.push_back(d.getAt2()); ia.push_back(d.getAt3()); ia.push_back(d.getAt4());
        it.push_back(d.getType()); iord.push_back(d.getOrder());
        ik.push_back(d.getK()); iph.push_back(d.getPhi0()); im.push_back(d.getMult());
    }
    mcg_system_desc d = {};
    d.natom = n;
    d.x = cx.data(); d.y = cy.data(); d.z = cz.data(); d.q = q.data();
    d.eps = eps.data(); d.sig = sig.data(); d.eps14 = eps14.data(); d.sig14 = sig14.data();
    d.mass = mass.data(); d.frozen = frozen.data(); d.resid = resid.data();
    switch (pbc.getType())
    {
    case NONE: d.pbc_type = MCG_PBC_NONE; break;
    case CUBIC: d.pbc_type = MCG_PBC_CUBIC; break;
    case ORBIC: d.pbc_type = MCG_PBC_ORBIC; break;
    default:
        std::cerr << "Error : FField_CUDA supports no, cubic and orthorhombic periodic boundaries" << std::endl;
        std::exit(-1);
    }
    pbc.get_pbc_vectors(d.box);
    d.cut_mode = cutMode == FULL ? MCG_CUT_FULL : MCG_CUT_SWITCH;
    d.cutoff = cutoff; d.cuton = cuton; d.dcut = deltacut;
    d.temp = ens.getTemp();
    d.precision = precision;
    d.nbond = (int)bt.size(); d.bond_atoms = ba.data(); d.bond_type = bt.data();
    d.bond_k = bk.data(); d.bond_r0 = br.data(); d.bond_beta = bb.data();
    d.nub = (int)uk.size(); d.ub_atoms = ua.data(); d.ub_k = uk.data(); d.ub_r0 = ur.data();
    d.nangle = (int)at.size(); d.angle_atoms = aa.data(); d.angle_type = at.data();
    d.angle_k = ak.data(); d.angle_theta0 = ath.data();
    d.ndihe = (int)dt.size(); d.dihe_atoms = da.data(); d.dihe_type = dt.data(); d.dihe_order = dord.data();
    d.dihe_k = dk.data(); d.dihe_phi0 = dph.data(); d.dihe_mult = dm.data();
    d.nimpr = (int)it.size(); d.impr_atoms = ia.data(); d.impr_type = it.data(); d.impr_order = iord.data();
    d.impr_k = ik.data(); d.impr_phi0 = iph.data(); d.impr_mult = im.data();
    d.param_units = MCG_UNITS_INTERNAL;
    if (cutMode == SHIFT)
    {
        std::cerr << "Error : FField_CUDA supports the 'full' and 'switch' cut modes" << std::endl;
        std::exit(-100);
    }
    check(mcg_create(&d, &sys), "create");
}

void FField_CUDA::upload()
{
    const int n = ens.getN();
    for (int i = 0; i < n; i++)
    {
        cx[i] = at_List.getX(i); cy[i] = at_List.getY(i); cz[i] = at_List.getZ(i);
    }
    check(mcg_set_coords(sys, cx.data(), cy.data(), cz.data()), "set_coords");
}

void FField_CUDA::compute()
{
    ensure();
    upload();
    double e[10];
    check(mcg_energy(sys, e), "energy");
    tot = e[0]; pot = e[1]; kin = e[2]; elec = e[3]; vdw = e[4];
    bond = e[5]; ang = e[6]; ub = e[7]; dihe = e[8]; impr = e[9];
}

double FField_CUDA::getE()
{
    ensure();
    double e = 0.0;
    check(mcg_energy_host(sys, at_List.getXvect().data(), at_List.getYvect().data(), at_List.getZvect().data(), &e),
          "energy_host");
    tot = pot = e;
    return tot;
}

void FField_CUDA::getE(double ener[10])
{
    compute();
    ener[0] = tot; ener[1] = pot; ener[2] = kin; ener[3] = elec; ener[4] = vdw;
    ener[5] = bond; ener[6] = ang; ener[7] = ub; ener[8] = dihe; ener[9] = impr;
}

void FField_CUDA::askListUpdate(int st)
{
    if (cutMode != FULL)
    {
        std::cout << "Verlet list updated at step " << st;
        auto start = std::chrono::system_clock::now();
        ensure();
        double e = 0.0;   // the device takes the AtomList's coordinates (commits an accepted move)
        check(mcg_energy_host(sys, at_List.getXvect().data(), at_List.getYvect().data(), at_List.getZvect().data(), &e),
              "energy_host");
        check(mcg_update_lists(sys), "update_lists");
        auto end = std::chrono::system_clock::now();
        std::cout << " : time required (milliseconds) : "
                  << std::chrono::duration_cast<std::chrono::milliseconds>(end - start).count() << std::endl;
    }
}

double FField_CUDA::getDeltaE(int n, const int* atoms, const double* x, const double* y, const double* z)
{
    ensure();
    upload();
    double de = 0.0;
    check(mcg_delta_e(sys, n, atoms, x, y, z, &de), "delta_e");
    return de;
}

// The component routines of the FField contract: the device computes all components in one pass.
double FField_CUDA::getEtot() { compute(); return tot; }
double FField_CUDA::getEswitch() { compute(); return tot; }
void FField_CUDA::computeNonBonded_full() { compute(); }
void FField_CUDA::computeNonBonded14() { compute(); }
void FField_CUDA::computeNonBonded_switch() { compute(); }
void FField_CUDA::computeNonBonded14_switch() { compute(); }
void FField_CUDA::computeEbond() { compute(); }
void FField_CUDA::computeEang() { compute(); }
void FField_CUDA::computeEub() { compute(); }
void FField_CUDA::computeEdihe() { compute(); }
void FField_CUDA::computeEimpr() { compute(); }
