// ref_probe — drives the compiled FHedin/mc_cpp reference (FField_MDBAS, List_nonBonded,
// MC machinery) to produce golden values for the oracle.  TEST INFRASTRUCTURE ONLY: built by
// oracle/ref.mk into oracle/_ref/, never shipped, never measured as the product.
//
// Modes (all energies in the reference's internal units, 1 kcal/mol = 418.4 iu):
//   ref_probe energy <xml>            one FField::getE(double[10]) as JSON     (FField_MDBAS.cpp:77-106)
//   ref_probe lists  <xml> <out.bin>  exclusion rows, 1-4 pairs, half Verlet rows (List_nonBonded.cpp:705-915)
//   ref_probe mc     <xml> <nsteps> <seed> <trace.bin>
//                                     Metropolis run with a per-step trace     (MC_metropolis.cpp:45-204)
//   ref_probe time   <xml> <reps>     wall time of getE() and update_verlet_list()
//
// The traced run restates MC_metropolis::run's draw order line for line (it has to be the same
// sequence to be a trace of it) and adds only logging.  The XML must set save_each="0".
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <chrono>
#include <vector>
#include <tuple>
#include <string>
#include <fcntl.h>
#include <unistd.h>

#include "Parser.hpp"
#include "PerConditions.hpp"
#include "Ensemble.hpp"
#include "AtomList.hpp"
#include "FField.hpp"
#include "List_nonBonded.hpp"
#include "List_Moves.hpp"
#include "MC.hpp"
#include "Move.hpp"
#include "Constants.hpp"

struct Loaded {
    PerConditions* pbc = nullptr;
    Ensemble* ens = nullptr;
    AtomList atoms;
    FField* ff = nullptr;
    List_nonBonded* lists = nullptr;
    List_Moves* moves = nullptr;
    MC* sim = nullptr;
};

static void load(const char* xml, Loaded& L)
{
    Parser_XML* p = new Parser_XML(xml, &L.pbc, &L.ens, L.atoms, &L.ff, &L.lists, &L.moves, &L.sim, false);
    delete p;
}

// One trace record per MC step: 12 doubles.
// st, imvtyp, imvatm, r0, r1, r2, rang, eold, enew, de, alpha(-1 if not drawn), accepted
class TracedMetropolis : public MC
{
public:
    TracedMetropolis(AtomList& a, PerConditions& p, Ensemble& e, FField& f, List_Moves& m,
                     int steps, uint64_t seed, FILE* out)
        : MC(a, p, e, f, m, steps, 0, seed), trace(out) {}

    void run() override
    {
        int nmvtyp = mvlist.getNMoveTypes();
        std::vector<int> nmvAccTmp(nmvtyp, 0);
        int natom = ens.getN();
        const std::vector<int>& nMoveAt = mvlist.getNMoveAtm();
        const std::vector<MOVETYPE>& movetypList = mvlist.getMoveTypeList();
        const std::vector<int**>& moveAtomList = mvlist.getMoveAtomList();
        const std::vector<int**>& movePivotList = mvlist.getMovePivotList();
        std::vector<std::tuple<double, double, double>> crdbackup(natom, std::tuple<double, double, double>(0.0, 0.0, 0.0));
        double etot = ff.getE();
        for (int st = 1; st <= nsteps; st++)
        {
            double rec[12] = {0};
            double r[3] = {0, 0, 0};
            double rang = 0.0;
            isAccepted = false;
            int imvtyp = rndIntCandidate(nmvtyp);
            int imvatm = rndIntCandidate(nMoveAt[imvtyp]);
            double eold = ff.getE();
            AtomList::crd_backup_save(crdbackup, at_List, moveAtomList[imvtyp][imvatm]);
            switch (movetypList[imvtyp])
            {
            case TRN:
                rndSphere(r);
                scaleVec(r, dmax[imvtyp]);
                rec[3] = r[0]; rec[4] = r[1]; rec[5] = r[2];
                MOVE_TRN::translate_set(at_List, pbc, moveAtomList[imvtyp][imvatm], r[0], r[1], r[2]);
                break;
            case ROT:
                rndSphere(r);
                rang = dmax[imvtyp] * rndUnifMove();
                rec[3] = r[0]; rec[4] = r[1]; rec[5] = r[2];
                MOVE_ROT::rotate_set(at_List, pbc, moveAtomList[imvtyp][imvatm],
                                     movePivotList[imvtyp][imvatm][0], rang, r);
                break;
            default:
                break;
            }
            double enew = ff.getE();
            double de = enew - eold;
            lastAlpha = -1.0;
            apply_criterion(de);
            if (isAccepted) { nmvAccTmp[imvtyp]++; etot += de; }
            else AtomList::crd_backup_load(crdbackup, at_List, moveAtomList[imvtyp][imvatm]);
            for (int iupdt = 0; iupdt < nmvtyp; iupdt++)
            {
                if (each[iupdt] != 0 && (st % each[iupdt]) == 0)
                {
                    adjust_dmax(dmax[iupdt], target[iupdt], each[iupdt], nmvAccTmp[iupdt]);
                    nmvAccTmp[iupdt] = 0;
                }
            }
            if (st % 50 == 0)
                lists->update_verlet_list();  // FField::askListUpdate without its timing printout
            rec[0] = st; rec[1] = imvtyp; rec[2] = imvatm; rec[6] = rang;
            rec[7] = eold; rec[8] = enew; rec[9] = de; rec[10] = lastAlpha; rec[11] = isAccepted ? 1.0 : 0.0;
            fwrite(rec, sizeof(double), 12, trace);
        }
        finalE = etot;
    }

    void apply_criterion(double de) override
    {
        const double dbl_epsilon = std::numeric_limits<double>::epsilon();
        if (de <= dbl_epsilon)
            isAccepted = true;
        else
        {
            double alpha = rndUnifAlpha();
            lastAlpha = alpha;
            double beta = 1.0 / ((CONSTANTS::rboltzui / CONSTANTS::kcaltoiu) * ens.getTemp());
            double accf = exp(-beta * de);
            isAccepted = (alpha < accf);
        }
    }

    List_nonBonded* lists = nullptr;
    double finalE = 0.0;

private:
    FILE* trace;
    double lastAlpha = -1.0;
};

static void write_ints(FILE* f, const std::vector<int>& v)
{
    int n = (int)v.size();
    fwrite(&n, sizeof(int), 1, f);
    if (n) fwrite(v.data(), sizeof(int), n, f);
}

int main(int argc, char** argv)
{
    if (argc < 3) { fprintf(stderr, "usage: ref_probe energy|lists|mc|time <xml> ...\n"); return 2; }
    std::string mode = argv[1];
    // The reference prints progress on stdout; keep stdout clean for the JSON result.
    fflush(stdout);
    int saved = dup(1);
    int devnull = open("/dev/null", O_WRONLY);
    dup2(devnull, 1);
    Loaded L;
    load(argv[2], L);
    std::cout.flush();
    fflush(stdout);
    dup2(saved, 1);
    close(saved);
    close(devnull);
    const int n = L.ens->getN();

    if (mode == "energy")
    {
        double e[10];
        L.ff->getE(e);
        long long listPairs = 0;
        if (L.ff->getCutMode() == SWITCH)
            for (int i = 0; i < n; i++) listPairs += L.lists->getNeighPair()[i];
        printf("{\"natom\": %d, \"ener\": [", n);
        for (int k = 0; k < 10; k++) printf("%s%.17g", k ? ", " : "", e[k]);
        printf("], \"list_pairs\": %lld}\n", listPairs);
    }
    else if (mode == "lists")
    {
        if (argc < 4) return 2;
        FILE* f = fopen(argv[3], "wb");
        // exclusion rows: exclPair[i] then the first exclPair[i] stored entries
        for (int i = 0; i < n; i++)
        {
            int c = L.lists->getExclPair()[i];
            std::vector<int> row(L.lists->getExclList()[i].begin(), L.lists->getExclList()[i].begin() + c);
            write_ints(f, row);
        }
        write_ints(f, L.lists->getNeighList14());
        bool sw = L.ff->getCutMode() == SWITCH;
        for (int i = 0; i < n; i++)
        {
            int c = sw ? L.lists->getNeighPair()[i] : 0;
            std::vector<int> row;
            if (c) row.assign(L.lists->getNeighList()[i].begin(), L.lists->getNeighList()[i].begin() + c);
            write_ints(f, row);
        }
        fclose(f);
    }
    else if (mode == "mc")
    {
        if (argc < 6) return 2;
        int nsteps = atoi(argv[3]);
        uint64_t seed = strtoull(argv[4], nullptr, 10);
        FILE* f = fopen(argv[5], "wb");
        std::cout.setstate(std::ios::failbit);
        TracedMetropolis mc(L.atoms, *L.pbc, *L.ens, *L.ff, *L.moves, nsteps, seed, f);
        mc.lists = L.lists;
        auto t0 = std::chrono::steady_clock::now();
        mc.run();
        auto t1 = std::chrono::steady_clock::now();
        std::cout.clear();
        fclose(f);
        printf("{\"nsteps\": %d, \"final_etot\": %.17g, \"seconds\": %.6f}\n", nsteps, mc.finalE,
               std::chrono::duration<double>(t1 - t0).count());
    }
    else if (mode == "time")
    {
        int reps = argc > 3 ? atoi(argv[3]) : 3;
        double e = 0;
        auto t0 = std::chrono::steady_clock::now();
        for (int r = 0; r < reps; r++) e += L.ff->getE();
        auto t1 = std::chrono::steady_clock::now();
        double tl = 0;
        if (L.ff->getCutMode() == SWITCH)
        {
            auto t2 = std::chrono::steady_clock::now();
            for (int r = 0; r < reps; r++) L.lists->update_verlet_list();
            auto t3 = std::chrono::steady_clock::now();
            tl = std::chrono::duration<double>(t3 - t2).count() / reps;
        }
        printf("{\"getE_s\": %.6g, \"list_s\": %.6g, \"e\": %.17g}\n",
               std::chrono::duration<double>(t1 - t0).count() / reps, tl, e / reps);
    }
    fflush(stdout);
    return 0;
}
