// adapter_check — builds the FField_CUDA adapter (mc_cpp_gb300/adapter/) inside the compiled
// FHedin/mc_cpp reference and runs it beside FField_MDBAS on one input.  TEST INFRASTRUCTURE
// ONLY: built by oracle/ref.mk into oracle/_ref/, never shipped, never measured.
//
//   adapter_check <xml> <cuton>   prints {"mdbas": [10 values], "cuda": [10 values]} (iu)
//
// The reference's Parser_XML builds the AtomList, PerConditions, Ensemble and an FField_MDBAS;
// FField_CUDA is then constructed on the same objects with the bonded lists copied through
// FField's public setters, as IO_MDBAS::read_ff would fill them (IO_MDBAS.cpp:490-503).  Without
// a GPU, FField_CUDA's first energy call exits through the reference's error convention.
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "Parser.hpp"
#include "FField.hpp"
#include "FField_CUDA.hpp"

int main(int argc, char** argv)
{
    if (argc < 3)
    {
        std::fprintf(stderr, "usage: adapter_check <xml> <cuton>\n");
        return 2;
    }
    PerConditions* pbc = nullptr;
    Ensemble* ens = nullptr;
    AtomList atoms;
    FField* ff = nullptr;
    List_nonBonded* lists = nullptr;
    List_Moves* moves = nullptr;
    MC* sim = nullptr;
    delete new Parser_XML(argv[1], &pbc, &ens, atoms, &ff, &lists, &moves, &sim, false);
    double ref[10];
    ff->getE(ref);

    const char* mode = ff->getCutMode() == FULL ? "full" : "switch";
    FField_CUDA cu(atoms, *pbc, *ens, mode, ff->getCutoff(), std::atof(argv[2]), ff->getDeltacut());
    std::vector<Bond> b(ff->getBndList());
    std::vector<Bond_UB> u(ff->getUbList());
    std::vector<Angle> a(ff->getAngList());
    std::vector<Dihedral> d(ff->getDiheList());
    std::vector<Dihedral_improper> im(ff->getImprList());
    cu.setBndList(b); cu.setNBond(ff->getNBond());
    cu.setUbList(u); cu.setNUb(ff->getNUb());
    cu.setAngList(a); cu.setNAngle(ff->getNAngle());
    cu.setDiheList(d); cu.setNDihedral(ff->getNDihedral());
    cu.setImprList(im); cu.setNImproper(ff->getNImproper());
    cu.setExcl(*lists);
    double got[10];
    cu.getE(got);
    std::printf("{\"mdbas\": [");
    for (int k = 0; k < 10; k++) std::printf("%s%.17g", k ? ", " : "", ref[k]);
    std::printf("], \"cuda\": [");
    for (int k = 0; k < 10; k++) std::printf("%s%.17g", k ? ", " : "", got[k]);
    std::printf("]}\n");
    return 0;
}
