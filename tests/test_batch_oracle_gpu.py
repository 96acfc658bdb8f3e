"""The batched sweep against an FP64 restatement of the same chains, move by move.

Each case builds a small batch, runs logged sweeps (the production sweep kernels, with per-move
records) and hands every chain's records to oracle/batch_oracle.cpp, which draws the same Philox
move in FP64, computes the FP64 dE of the recorded proposal over every atom pair within the cutoff,
decides with the reference's criterion (MC_metropolis.cpp:175-204) and then follows the recorded
decision.  Checked per move:

* the recorded residue, move type and acceptance draw are the ones the chain's Philox stream gives;
* the recorded proposal is the FP64 move within 1e-5 A (the device forms moves in FP32);
* |dE_mixed - dE_FP64| <= 1e-4 kcal/mol (the mixed-precision target);
* the recorded decision is the reference's criterion applied to the recorded dE and draw;
* where the FP64 decision differs from it, the draw lies between the two acceptance thresholds
  exp(-beta dE) (a tie that the dE error decides), with |alpha - exp(-beta dE_FP64)| bounded by
  what a 1e-4 kcal/mol error can move the threshold;
and per sweep: the device coordinates equal the restatement's (the accepted moves were committed
and nothing else), the running energy equals the FP64 start energy plus the FP64 dE of the
accepted moves, and the device's FP64 recompute equals the restatement's total.

Cases: the tuner's launch shape on water chains of 512-8192 molecules (the largest on a two-CTA
cluster), one-CTA chains with speculation 8 and dmax adjustment, chains with speculation 16 (one
of them on a two-CTA cluster), and argon chains (translations only).
"""
import json
import os
import sys

import numpy as np
import pytest

from mc_cpp_gb300 import build, native, systems
from mc_cpp_gb300.engine import BatchChains

sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle"))
import oracle as orc  # noqa: E402

pytestmark = pytest.mark.gpu
KCAL = 418.4
DE_TOL_KCAL = 1e-4
POS_TOL = 1e-5
SEED = 77

CASES = {
    # tuned launch shape; the 8192-molecule chain runs on a two-CTA cluster when clusters are on
    "water_tuned": dict(chains=lambda: [systems.water_box(8192, seed=41, temp=300.0),
                                        systems.water_box(512, seed=42, temp=285.0),
                                        systems.water_box(2000, seed=43, temp=355.0)],
                        opts=dict(dmax_trn=0.15, dmax_rot=15.0), tune=True, sweeps=2),
    "water_spec8_dmax": dict(chains=lambda: [systems.water_box(600, seed=44, temp=280.0),
                                             systems.water_box(1500, seed=45, temp=320.0),
                                             systems.water_box(3000, seed=46, temp=360.0)],
                             opts=dict(dmax_trn=0.15, dmax_rot=15.0, clusters=-1, speculation=8, threads_per_chain=256,
                                       dmax_each=(40, 40), dmax_target=(40.0, 40.0)), tune=False, sweeps=2),
    # 16 moves per iteration: one warp per move on one CTA, two warps per move on a two-CTA cluster;
    # in the 600-molecule box every pair of moves of an iteration may interact
    "water_spec16": dict(chains=lambda: [systems.water_box(600, seed=47, temp=300.0),
                                         systems.water_box(1300, seed=48, temp=330.0),
                                         systems.water_box(4000, seed=49, temp=290.0)],
                         opts=dict(dmax_trn=0.15, dmax_rot=15.0, clusters=0, speculation=16, threads_per_chain=512),
                         tune=False, sweeps=2),
    "argon": dict(chains=lambda: [systems.argon_random(700, 0.02, 51, temp=120.0),
                                  systems.argon_random(1900, 0.016, 52, temp=95.0)],
                  opts=dict(dmax_trn=0.2, dmax_rot=0.0, clusters=-1), tune=False, sweeps=2),
}


@pytest.fixture(scope="module", autouse=True)
def _built():
    build.build()
    orc.build()
    if native.lib().mcg_device_count() < 1:
        pytest.fail("no CUDA device visible to libmcgpu.so")


def _mic(a, b, box):
    d = a - b
    return d - box * np.round(d / box)


@pytest.mark.parametrize("case", sorted(CASES))
def test_batched_chain_follows_the_fp64_restatement(case):
    spec = CASES[case]
    chains = spec["chains"]()
    o = dict(spec["opts"])
    B = BatchChains(chains, acceptance="physical", seed=SEED, **o)
    tuning = B.autotune(trial_sweeps=1, use_cache=False) if spec["tune"] else B.tuning()
    trials0, _, _ = B.stats()
    each = o.get("dmax_each", (0, 0))
    orcs = []
    for k, s in enumerate(chains):
        t = s.copy()
        t.set_coords(B.coords(k))
        oc = orc.BatchChainOracle(t, chain=k, seed=SEED, dmax=(o["dmax_trn"], o["dmax_rot"]), each=each,
                                  target=o.get("dmax_target", (50.0, 50.0)))
        oc.set_moves(int(trials0[k]))
        orcs.append(oc)
    e_start = np.array([oc.energy() for oc in orcs])
    _, _, etot0 = B.stats()
    # the running energy after the tuner's sweeps is the FP64 energy of the same coordinates
    for k in range(len(chains)):
        assert abs(etot0[k] - e_start[k]) <= 1e-6 * max(abs(e_start[k]), 10 * KCAL * chains[k].natom / 3)
    acc_de64 = np.zeros(len(chains))
    summary = {"case": case, "tuning": tuning, "chains": []}
    for sweep in range(spec["sweeps"]):
        recs = B.sweep_logged()
        for k, (oc, rec) in enumerate(zip(orcs, recs)):
            r = oc.follow(rec)
            n = len(rec)
            dev_acc = (rec["flags"] & 2) != 0
            assert r["match"].all(), "chain %d: residue or move type differs from the Philox draw at %s" % (
                k, np.nonzero(r["match"] == 0)[0][:5])
            assert r["alpha_match"].all(), "chain %d: acceptance draws differ" % k
            assert np.nanmax(r["pos_err"]) <= POS_TOL, (k, np.nanmax(r["pos_err"]))
            de_err = np.abs(rec["de"] - r["de64"]) / KCAL
            assert de_err.max() <= DE_TOL_KCAL, (k, de_err.max(), int(de_err.argmax()))
            # the device applied the reference's criterion to its own dE and draw, exactly
            assert np.array_equal(r["acc_rule"] != 0, dev_acc), (k, np.nonzero((r["acc_rule"] != 0) != dev_acc)[0][:5])
            mism = np.nonzero((r["acc64"] != 0) != dev_acc)[0]
            beta = 1.0 / (0.0019872 * chains[k].temp)              # mol/kcal, physical units
            gap = np.abs(r["alpha"][mism] - r["thr64"][mism])
            assert (gap <= beta * DE_TOL_KCAL * 1.01 + 1e-12).all(), (k, mism, gap)
            assert len(mism) <= max(1, n // 1000), (k, len(mism))
            acc_de64[k] += r["de64"][dev_acc].sum()
            # the device committed exactly the accepted proposals
            box = np.array(chains[k].box if chains[k].pbc_type == "orbic" else (chains[k].box[0],) * 3)
            assert np.abs(_mic(B.coords(k), oc.coords(), box)).max() <= 1e-9
            summary["chains"].append({"chain": k, "sweep": sweep, "moves": n, "accepted": int(dev_acc.sum()),
                                      "max_dE_err_kcal_mol": float(de_err.max()),
                                      "rms_dE_err_kcal_mol": float(np.sqrt((de_err ** 2).mean())),
                                      "max_pos_err_A": float(np.nanmax(r["pos_err"])),
                                      "decision_ties": int(len(mism)),
                                      "max_tie_gap": float(gap.max()) if len(mism) else 0.0})
    _, _, etot = B.stats()
    e64 = B.energy_fp64()
    for k, oc in enumerate(orcs):
        e_end = oc.energy()
        scale = max(abs(e_end), 10 * KCAL * chains[k].natom / 3)
        assert abs(e64[k] - e_end) <= 1e-10 * scale, (k, e64[k], e_end)
        assert abs(etot[k] - (e_start[k] + acc_de64[k])) <= 1e-6 * scale, (k, etot[k], e_start[k] + acc_de64[k])
        assert abs(etot[k] - e_end) <= 1e-6 * scale, (k, etot[k], e_end)
        if each[0] or each[1]:
            dt, dr = B.dmax()
            assert np.allclose(oc.dmax(), [dt[k], dr[k]], rtol=1e-12, atol=0)
    print("BATCH_ORACLE " + json.dumps(summary))
    B.close()


def test_headline_shape_batch_against_the_restatement():
    """The benchmark's chain generator (fewer chains) plus its extreme sizes, 512 and 8192
    molecules, at the launch shape the tuner picks: after two sweeps every chain's FP64 recompute
    equals the restatement's energy of the same coordinates, and every running energy equals it."""
    chains = systems.water_chains(nchains=10, seed=3) + [systems.water_box(512, seed=61, temp=300.0),
                                                         systems.water_box(8192, seed=62, temp=330.0)]
    B = BatchChains(chains, dmax_trn=0.15, dmax_rot=15.0, acceptance="physical", seed=5)
    tuning = B.autotune(trial_sweeps=1, use_cache=False)
    B.sweep(2)
    _, acc, etot = B.stats()
    e64 = B.energy_fp64()
    assert (acc > 0).all()
    for k, s in enumerate(chains):
        t = s.copy()
        t.set_coords(B.coords(k))
        want = orc.BatchChainOracle(t, chain=k, seed=5).energy()
        scale = max(abs(want), 10 * KCAL * s.natom / 3)
        assert abs(e64[k] - want) <= 1e-10 * scale, (k, e64[k], want)
        assert abs(etot[k] - want) <= 1e-6 * scale, (k, etot[k], want)
    print("HEADLINE_SHAPE " + json.dumps({"tuning": tuning, "sizes": [int(s.natom // 3) for s in chains]}))
    B.close()
