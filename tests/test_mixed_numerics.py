"""A float32 restatement of the mixed pair kernel's arithmetic (numpy), against the FP64 oracle.

k_energy_list_mix (mc_cpp_gb300/csrc/single.cu) forms each displacement exactly as a 32-bit
fixed-point difference (box = 2^32 units, wrap-around = minimum image), sums r^2 in FP32 units and
scales it by the float-float square of the unit length (cubic boxes), and evaluates the switched
Coulomb and LJ terms in FP32: the switch as (rc^2 - u)^2 (2u + rc^2 - 3 ron^2) with
u = max(r^2, ron^2), normalised once by its value at ron^2; per lane and row, q_j S/r summed in
float-float and eps_j (x^12 - x^6) S summed in FP32 (lane = entry index mod 32), multiplied by
q_i and eps_i at the row's end.  This restatement runs the same arithmetic in numpy float32 (an FMA
is emulated as one float64 product-sum rounded once to float32; 1/sqrt as the correctly rounded
float32 value, within 2 ulp of the kernel's rsqrt + Newton step) over the oracle's Verlet rows.

It checks the design, not the device: the total energy within 1e-6 relative of the oracle's FP64
value (the tolerance the GPU tests apply to the kernel), each component within 1e-6 of the larger
of the two.  The packed group-pair kernels' arithmetic (partners placed relative to the row
group's first atom, the switch as a polynomial in rc^2 - r^2, the inverse distance scaled by -2)
is restated the same way (packed_energy): 2.6e-8 to 8.8e-8 of the larger component on argon,
water 512 and water 4,096, as the list kernel's restatement.
"""
import math

import numpy as np
import pytest

import goldens
import oracle as orc

KCALTOIU = 418.4
CHGCHARMM = 332.0716
TOL = 1e-6
f32 = np.float32


def _fma(a, b, c):
    return (a.astype(np.float64) * b.astype(np.float64) + np.asarray(c, np.float64)).astype(f32)


def _to_fixed(x, L):
    u = x / L
    u = u - np.rint(u)                                       # [-0.5, 0.5]
    v = np.rint(u * 4294967296.0).astype(np.int64)
    return (v & 0xFFFFFFFF).astype(np.uint32)


def mixed_energy(s, rows, scale_lo=True):
    """(elec, vdw) in internal units, by the kernel's arithmetic in float32.  scale_lo=False drops
    the low part of the squared unit length: a float-rounded scale, for the test below."""
    L = float(s.box[0])
    assert s.box[0] == s.box[1] == s.box[2], "cubic boxes (the kernel's ISO path)"
    n = s.natom
    i = np.repeat(np.arange(n), [len(r) for r in rows])
    j = np.concatenate(rows).astype(np.int64)
    k = np.concatenate([np.arange(len(r)) for r in rows])   # entry index within its row
    fx = [_to_fixed(np.asarray(c, np.float64), L) for c in (s.x, s.y, s.z)]
    # the unit length L / 2^32 as a float-float pair, and its square as a float-float pair
    ls = L / 4294967296.0
    lh = f32(ls)
    ll = f32(ls - float(lh))
    l2 = (float(lh) + float(ll)) ** 2
    L2h = f32(l2)
    L2l = f32(l2 - float(L2h)) if scale_lo else f32(0.0)
    u = [(fx[a][j] - fx[a][i]).astype(np.uint32).view(np.int32).astype(f32) for a in range(3)]
    r2u = _fma(u[0], u[0], _fma(u[1], u[1], u[2] * u[2]))
    r2 = _fma(r2u, np.full_like(r2u, L2h), r2u * L2l)
    c2, n2 = f32(s.cutoff * s.cutoff), f32(s.cuton * s.cuton)
    k3 = f32(c2 - f32(3.0) * n2)
    inside = r2 <= c2
    i, j, k, r2 = i[inside], j[inside], k[inside], r2[inside]
    rinv = (1.0 / np.sqrt(r2.astype(np.float64))).astype(f32)
    uu = np.maximum(r2, n2)
    a = (c2 - uu).astype(f32)
    f = (a * a * _fma(np.full_like(uu, 2.0), uu, k3)).astype(f32)
    g = (rinv * f).astype(f32)
    # per-atom parameters as the kernel holds them
    q = np.asarray(s.q, np.float64)
    qh = q.astype(f32)
    ql = (q - qh.astype(np.float64)).astype(f32)
    eps = np.sqrt(np.asarray(s.eps, np.float64) * KCALTOIU).astype(f32)
    sig = np.asarray(s.sig, np.float64).astype(f32)
    # Coulomb: q_j g summed per (row, lane) in float-float (~exact: float64 sums of FP32 products)
    lane = i * 32 + (k % 32)
    ce = np.zeros(32 * n, np.float64)
    np.add.at(ce, lane, (qh[j] * g).astype(np.float64) + (ql[j] * g).astype(np.float64))
    # LJ: eps_j (x^12 - x^6) f summed per (row, lane) in FP32, in entry order
    y = ((sig[i] + sig[j]) * rinv).astype(f32)
    x2 = (y * y).astype(f32)
    x6 = (x2 * x2 * x2).astype(f32)
    term = (eps[j] * (_fma(x6, x6, -x6) * f).astype(f32)).astype(f32)
    ve = np.zeros(32 * n, f32)
    np.add.at(ve, lane, term)
    # row flush: q_i (float-float) and eps_i, then the normalisation of the switch
    rowq = (qh.astype(np.float64) + ql.astype(np.float64))[np.arange(32 * n) // 32]
    rowe = eps.astype(np.float64)[np.arange(32 * n) // 32]
    a1 = float(c2 - n2)
    f1 = float(f32(f32(a1 * a1) * _fma(np.array([2.0], f32), np.array([n2], f32), k3)[0]))
    elec = float(np.sum(rowq * ce)) / f1
    vdw = float(np.sum(rowe * ve.astype(np.float64))) / f1
    return CHGCHARMM * KCALTOIU * elec, 4.0 * vdw


@pytest.fixture(scope="module", autouse=True)
def _built():
    orc.build()


@pytest.mark.parametrize("name", ["argon864", "water512", "water4096"])
def test_mixed_arithmetic_within_tolerance_of_fp64(name):
    s = goldens.system(name, "switch")
    o = orc.Oracle(s, moves=False)
    want = o.energy()
    elec, vdw = mixed_energy(s, o.verlet_rows())
    scale = max(1.0, abs(want[3]), abs(want[4]))
    assert abs(elec - want[3]) <= TOL * scale, (elec, want[3])
    assert abs(vdw - want[4]) <= TOL * scale, (vdw, want[4])
    assert abs((elec + vdw) - (want[3] + want[4])) <= TOL * max(1.0, abs(want[3] + want[4])), (elec + vdw, want)


def test_float_float_scale_removes_the_scale_bias():
    """Why the unit length is a float-float pair: rounded to one float, the scale stretches every
    distance by the same factor, and the unrelaxed box's virial turns that into a total-energy
    error several times larger (water, 12,288 atoms: ~8e-8 with the pair, ~7e-7 without)."""
    s = goldens.system("water4096", "switch")
    o = orc.Oracle(s, moves=False)
    want = o.energy()
    rows = o.verlet_rows()
    tot = want[3] + want[4]
    err_ff = abs(sum(mixed_energy(s, rows)) - tot) / abs(tot)
    err_f = abs(sum(mixed_energy(s, rows, scale_lo=False)) - tot) / abs(tot)
    assert err_ff <= 2e-7, err_ff
    assert err_f >= 3.0 * err_ff, (err_f, err_ff)


def _pair_delta(do, m, qk_sw, e4_sw, ss, c2, n2, k3):
    """mixed_pair_delta_clamped (mc_cpp_gb300/csrc/pair_math.cuh) in numpy float32: the energy
    change of pairs whose first atom moves by m (d_new = d_old - m), Coulomb differenced
    analytically.  Arrays of shape (npairs, 3) / (npairs,)."""
    dn = (do - m).astype(f32)
    uo = _fma(do[:, 0], do[:, 0], _fma(do[:, 1], do[:, 1], do[:, 2] * do[:, 2]))
    un = _fma(dn[:, 0], dn[:, 0], _fma(dn[:, 1], dn[:, 1], dn[:, 2] * dn[:, 2]))
    ro = (1.0 / np.sqrt(uo.astype(np.float64))).astype(f32)
    rn = (1.0 / np.sqrt(un.astype(np.float64))).astype(f32)
    ua = np.minimum(np.maximum(uo, n2), c2)
    ub = np.minimum(np.maximum(un, n2), c2)
    Aa, Ab = (c2 - ua).astype(f32), (c2 - ub).astype(f32)
    two = np.full_like(ua, 2.0)
    Ba, Bb = _fma(two, ua, k3), _fma(two, ub, k3)
    po, pn = (Aa * Aa * Ba).astype(f32), (Ab * Ab * Bb).astype(f32)
    xo, xn = (ss * (ro * ro)).astype(f32), (ss * (rn * rn)).astype(f32)
    xo3, xn3 = (xo * xo * xo).astype(f32), (xn * xn * xn).astype(f32)
    d_lj = (e4_sw * _fma(_fma(xn3, xn3, -xn3), pn, -(_fma(xo3, xo3, -xo3) * po))).astype(f32)
    s = (do + dn).astype(f32)
    du = -_fma(m[:, 0], s[:, 0], _fma(m[:, 1], s[:, 1], m[:, 2] * s[:, 2]))
    p = (ro * rn).astype(f32)
    dinv = ((-du * p * p).astype(f32) / (ro + rn).astype(f32)).astype(f32)
    dd = np.where((ua == uo) & (ub == un), du, (ub - ua).astype(f32))
    dp = (dd * _fma((two * Aa).astype(f32), Aa, -((Aa + Ab) * Bb).astype(f32))).astype(f32)
    return _fma(qk_sw, _fma(dinv, pn, (ro * dp).astype(f32)), d_lj)


def _pair_direct(d, qk_sw, e4_sw, ss, c2, n2, k3):
    """The same pair energy evaluated directly in float32 (for the comparison below)."""
    u = _fma(d[:, 0], d[:, 0], _fma(d[:, 1], d[:, 1], d[:, 2] * d[:, 2]))
    r = (1.0 / np.sqrt(u.astype(np.float64))).astype(f32)
    uc = np.minimum(np.maximum(u, n2), c2)
    A = (c2 - uc).astype(f32)
    P = (A * A * _fma(np.full_like(uc, 2.0), uc, k3)).astype(f32)
    x = (ss * (r * r)).astype(f32)
    x3 = (x * x * x).astype(f32)
    return (qk_sw * (r * P).astype(f32) + e4_sw * (_fma(x3, x3, -x3) * P).astype(f32)).astype(f32)


def test_mixed_delta_e_within_tolerance_and_analytic_coulomb_difference():
    """Residue moves of the 12,288-atom water box (translations <= 0.15 A, rotations <= 15 deg
    about the oxygen): the float32 dE over the moved atoms' Verlet partners against the oracle's
    FP64 dE.  The analytic Coulomb difference keeps every dE within 1e-4 kcal/mol; the pair
    energies differenced directly in float32 would err several times more."""
    s = goldens.system("water4096", "switch")
    o = orc.Oracle(s, moves=False)
    rows = o.verlet_rows()
    pi = np.repeat(np.arange(s.natom), [len(r) for r in rows])
    pj = np.concatenate(rows).astype(np.int64)
    L = float(s.box[0])
    fx = np.stack([_to_fixed(np.asarray(c, np.float64), L) for c in (s.x, s.y, s.z)], 1)
    ls = L / 4294967296.0
    lh = f32(ls)
    ll = f32(ls - float(lh))
    c2, n2 = f32(s.cutoff * s.cutoff), f32(s.cuton * s.cuton)
    k3 = f32(c2 - f32(3.0) * n2)
    sw2 = f32(1.0 / (float(s.cutoff) ** 2 - float(s.cuton) ** 2) ** 3)
    q = np.asarray(s.q, np.float64)
    eps = np.sqrt(np.asarray(s.eps, np.float64) * KCALTOIU).astype(f32)
    sig = np.asarray(s.sig, np.float64).astype(f32)
    xyz = s.coords()
    rng = np.random.default_rng(21)
    worst_a, worst_d = 0.0, 0.0
    for t in range(24):
        r = int(rng.integers(0, 4096))
        idx = np.arange(3 * r, 3 * r + 3)
        if t % 2 == 0:
            v = rng.normal(size=3)
            new = xyz[idx] + 0.15 * rng.uniform() ** (1 / 3) * v / np.linalg.norm(v)
        else:
            ax = rng.normal(size=3)
            ax /= np.linalg.norm(ax)
            th = np.radians(rng.uniform(-15.0, 15.0))
            K = np.array([[0, -ax[2], ax[1]], [ax[2], 0, -ax[0]], [-ax[1], ax[0], 0]])
            R = np.eye(3) + np.sin(th) * K + (1 - np.cos(th)) * K @ K
            new = xyz[idx[0]] + (xyz[idx] - xyz[idx[0]]) @ R.T
        want = o.delta_e(idx, new)
        da, dd = 0.0, 0.0
        for k, a in enumerate(idx):
            sel = (pi == a) | (pj == a)
            other = np.where(pi[sel] == a, pj[sel], pi[sel])
            other = other[(other < idx[0]) | (other > idx[-1])]
            f = (fx[other].astype(np.int64) - fx[a].astype(np.int64)).astype(np.uint32).view(np.int32).astype(f32)
            do = _fma(f, np.full_like(f, lh), f * ll)                       # fixed_delta, per axis
            m = np.broadcast_to((new[k] - xyz[a]).astype(f32), do.shape).astype(f32)
            qk_sw = (CHGCHARMM * KCALTOIU * q[a] * q[other]).astype(f32) * sw2
            e4_sw = (f32(4.0) * eps[a] * eps[other]).astype(f32) * sw2
            ss = ((sig[a] + sig[other]) ** 2).astype(f32)
            da += float(np.sum(_pair_delta(do, m, qk_sw, e4_sw, ss, c2, n2, k3).astype(np.float64)))
            dn = (do - m).astype(f32)
            dd += float(np.sum(_pair_direct(dn, qk_sw, e4_sw, ss, c2, n2, k3).astype(np.float64)
                               - _pair_direct(do, qk_sw, e4_sw, ss, c2, n2, k3).astype(np.float64)))
        worst_a = max(worst_a, abs(da - want) / KCALTOIU)
        worst_d = max(worst_d, abs(dd - want) / KCALTOIU)
    assert worst_a <= 1e-4, worst_a
    assert worst_d >= 3.0 * worst_a, (worst_d, worst_a)


def test_packed_switch_polynomial_in_u_equals_the_reference_switch():
    """The packed group-pair kernels (k_energy_groups_x2*, mc_cpp_gb300/csrc/groups.cu) evaluate the
    switch as P = u^2 (3D - 2u) on u = clamp(rc^2 - r^2, 0, D), D = rc^2 - ron^2, in float32, and
    divide the block sums by P(D) in FP64.  The reference's switch is
    (rc^2 - r^2)^2 (rc^2 + 2 r^2 - 3 ron^2) / (rc^2 - ron^2)^3 between ron and rc, 1 below, 0
    beyond (FField_MDBAS.cpp:348-402).  Checked on r from 0.5 to 13 A for the 10-12 and 8-9 A switches: within 4 float32
    roundings of the FP64 value, exactly 1 below ron (P(D) is formed as the kernel forms it) and
    exactly 0 beyond rc."""
    for ron, rc in ((10.0, 12.0), (8.0, 9.0)):
        c2, n2 = f32(rc * rc), f32(ron * ron)
        D = f32(c2 - n2)
        d3 = f32(f32(3.0) * D)
        r = np.linspace(0.5, 13.0, 20001)
        r2 = (r * r).astype(f32)
        u = np.minimum(np.maximum((c2 - r2).astype(f32), f32(0.0)), D)
        P = ((u * u).astype(f32) * _fma(u, np.full_like(u, -2.0), d3)).astype(f32)
        pD = float(f32(D * D) * _fma(np.array([D]), np.array([f32(-2.0)]), d3)[0])
        S = P.astype(np.float64) / pD
        r2d = r2.astype(np.float64)
        c2d, n2d = float(c2), float(n2)
        ref = np.where(r2d <= n2d, 1.0, np.where(r2d >= c2d, 0.0,
                       (c2d - r2d) ** 2 * (c2d + 2.0 * r2d - 3.0 * n2d) / (c2d - n2d) ** 3))
        assert np.all(S[r2d <= n2d] == 1.0)
        assert np.all(S[r2d >= c2d] == 0.0)
        mid = (r2d > n2d) & (r2d < c2d)
        assert np.all(np.abs(S[mid] - ref[mid]) <= 4 * 2.0 ** -24 * np.maximum(ref[mid], 2.0 ** -20))


def _fixed_delta(fa, fb, lh, ll):
    """fixed_delta (pair_math.cuh): the int32 wrap of b - a converted to float32 and scaled by the
    float-float unit length."""
    f = (fb - fa).astype(np.uint32).view(np.int32).astype(f32)
    return _fma(f, np.full_like(f, lh), (f * ll).astype(f32))


def packed_energy(s, rows):
    """(elec, vdw) in internal units by the pair arithmetic of the packed group-pair kernels
    (k_energy_groups_x2*, mc_cpp_gb300/csrc/groups.cu), in float32; pair terms summed in float64
    (the kernels' float-float row sums are the other test's subject).  Groups are runs of up to 4
    atoms of one residue; a row group of G atoms whose offsets from its first atom stay within
    emax places its partners relative to that atom and adds each row atom's own offset, the other
    rows take the per-pair displacement.  The switch is u^2 (3D - 2u), u = clamp(rc^2 - r^2, 0, D);
    the inverse distance carries a factor -2 (exact) that the Coulomb sums drop at the row's end
    and the half sigmas carry as -1/2."""
    L = [float(b) for b in s.box]
    n = s.natom
    resid = np.asarray(s.resid)
    gstart = []
    for a in range(n):
        if a == 0 or resid[a] != resid[a - 1] or a - gstart[-1] == 4:
            gstart.append(a)
    gof = np.repeat(np.arange(len(gstart)), np.diff(gstart + [n]))
    first = np.asarray(gstart)[gof]
    gsize = np.diff(gstart + [n])
    G = 3 if gsize.max() <= 3 else 4
    i = np.repeat(np.arange(n), [len(r) for r in rows])
    j = np.concatenate(rows).astype(np.int64)
    fx, lh, ll = [], [], []
    for a in range(3):
        fx.append(_to_fixed(np.asarray((s.x, s.y, s.z)[a], np.float64), L[a]))
        ls = L[a] / 4294967296.0
        lh.append(f32(ls))
        ll.append(f32(ls - float(f32(ls))))
    c2, n2 = f32(s.cutoff * s.cutoff), f32(s.cuton * s.cuton)
    D = f32(c2 - n2)
    emax = f32(0.5 * min(L) - math.sqrt(float(c2)) - 1e-3)
    # each atom's offset from its group's first atom, and the row groups that take the relative form
    off = [_fixed_delta(fx[a][first], fx[a], lh[a], ll[a]) for a in range(3)]
    big = np.maximum.reduce([np.abs(o) for o in off])
    gbig = np.zeros(len(gstart), f32)
    np.maximum.at(gbig, gof, big)
    rel = (gsize[gof[i]] == G) & (gbig[gof[i]] <= emax)
    d = []
    for a in range(3):
        dj = _fixed_delta(fx[a][first[i]], fx[a][j], lh[a], ll[a])
        d_rel = (dj + (-off[a][i])).astype(f32)
        d_pair = _fixed_delta(fx[a][i], fx[a][j], lh[a], ll[a])
        d.append(np.where(rel, d_rel, d_pair))
    r2 = _fma(d[0], d[0], _fma(d[1], d[1], (d[2] * d[2]).astype(f32)))
    u = np.minimum(np.maximum((c2 - r2).astype(f32), f32(0.0)), D)
    P = ((u * u).astype(f32) * _fma(u, np.full_like(u, -2.0), np.full_like(u, f32(3.0) * D))).astype(f32)
    ri = (f32(-2.0) * (1.0 / np.sqrt(r2.astype(np.float64))).astype(f32)).astype(f32)
    gg = (ri * P).astype(f32)
    q = np.asarray(s.q, np.float64)
    qh = q.astype(f32)
    ql = (q - qh.astype(np.float64)).astype(f32)
    eps = np.sqrt(np.asarray(s.eps, np.float64) * KCALTOIU).astype(f32)
    hs = (f32(-0.5) * np.asarray(s.sig, np.float64).astype(f32)).astype(f32)
    y = ((hs[i] + hs[j]) * ri).astype(f32)
    x2 = (y * y).astype(f32)
    x6 = (x2 * x2 * x2).astype(f32)
    lj = (eps[j] * ((_fma(x6, x6, -x6) * P).astype(f32))).astype(f32)
    cq = (qh[j] * gg).astype(np.float64) + (ql[j] * gg).astype(np.float64)
    pD = float(f32(D * D) * _fma(np.array([D]), np.array([f32(-2.0)]), np.array([f32(3.0) * D]))[0])
    elec = -0.5 * float(np.sum(q[i] * cq)) / pD
    vdw = float(np.sum(eps[i].astype(np.float64) * lj.astype(np.float64))) / pD
    return CHGCHARMM * KCALTOIU * elec, 4.0 * vdw, float(np.mean(rel))


@pytest.mark.parametrize("name", ["argon864", "water512", "water4096"])
def test_packed_group_arithmetic_within_tolerance_of_fp64(name):
    """The packed kernels' pair arithmetic (relative placement, switch in u, the -2 scaled inverse
    distance) in float32 against the oracle's FP64 energy: within 1e-6 of the larger component, as
    the GPU tests hold the kernels.  water4096 takes the relative placement on every row, water512
    (half the box less rc below the hydrogens' offsets) and argon (one-atom groups) the per-pair
    displacement."""
    s = goldens.system(name, "switch")
    o = orc.Oracle(s, moves=False)
    want = o.energy()
    elec, vdw, frac_rel = packed_energy(s, o.verlet_rows())
    assert frac_rel == {"argon864": 0.0, "water512": 0.0, "water4096": 1.0}[name], frac_rel
    scale = max(1.0, abs(want[3]), abs(want[4]))
    assert abs(elec - want[3]) <= TOL * scale, (elec, want[3])
    assert abs(vdw - want[4]) <= TOL * scale, (vdw, want[4])
