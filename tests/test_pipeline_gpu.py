"""End-to-end pins against the reference's own example runs (golden eval.dat).

The whole filter path runs on the GPU -- spectrum range, Newton
coefficients, random starts, Newton filter, orthogonalisation, subspace
diagonalisation, sigma_E -- on the reference's example inputs (conf.par,
pot*.par, SO_*.par, input.par), in FP64 and in the mixed path (FP32 recursion
and FFTs, FP64 accumulators and eigensolves).  The reference's starts were
clock-seeded, so the filtered subspaces differ; converged eigenvalues must
agree to 1e-5 Ha.  The mixed path's converged eigenvectors must span the FP64
path's degenerate eigenspaces on the same starts."""
import os

import numpy as np
import pytest

from oracle import oracle as O
from tests.systems import GOLD, read_conf, read_pot

pytestmark = pytest.mark.gpu

# sigma_E below which our pairs are matched to the reference's converged
# levels: the FP64 path converges them to 1e-4; the mixed path's FP32
# recursion leaves noise of about 1e-4 of the norm in every filtered state,
# spread over the whole spectrum, so its residuals stay near 1e-3 while its
# energies (second order in that noise) still match -- its pairs are taken up
# to the reference's own sigmaECut (filter_mpi/read.c:86)
MY_SIGMA = {0: 1e-4, 1: 1e-2}


def _targets(vbmin, vbmax, cbmin, cbmax, nvb, ncb):
    return O.ene_targets(vbmin, vbmax, cbmin, cbmax, nvb, ncb)


def _run(fbse, cuda, grid, pot, targets, ncheby, nstart, nspin, cplx, so=False, nl=False, proj=None, seed=-31415,
         precision=0, states=False):
    import torch
    ctx = fbse.Context(grid, pot, nspin=nspin, is_complex=cplx, so=so, nl=nl, proj=proj, precision=precision)
    e0, e1, it = ctx.energy_range()
    emin = e0 - 0.2 * abs(e0)  # energy.c:360-363 (SO or no projectors)
    emax = e1 * 1.2
    de = emax - emin
    zn, _ = fbse.samp_points(ncheby)
    an = fbse.newton_coeff(zn, targets, emin, de, O.filter_dt(ncheby, de))
    starts, _, _ = fbse.init_filter_states(nstart, grid.ngrid, nspin, cplx, grid.dv, seed)
    filt = ctx.newton_filter(zn, an, emin, de, torch.tensor(starts, device=cuda))
    m = len(targets)
    psitot = filt.reshape(nstart * m, -1)
    nk, ev, sg = ctx.ortho_diag_sigma(psitot)
    if states:
        return (emin, emax), ev, sg, psitot[:nk].cpu().numpy()
    return (emin, emax), ev, sg


def _match(ref, ev, sg, ref_sig, my_sig, tol):
    r = ref[ref[:, 2] < ref_sig]
    mine = ev[sg < my_sig]
    d = np.array([np.min(np.abs(mine - e)) if len(mine) else np.inf for e in r[:, 1]])
    return r, d


@pytest.mark.parametrize("precision", [0, 1])
def test_cdse22_real_matches_reference_eval(fbse, cuda, precision):
    """2.2 nm CdSe, real, 57 x 52 x 45 at 0.8 bohr, 16 starts (FP64; 48 mixed) x 16 targets,
    nCheby 2048 (filter_mpi/EXAMPLES/2.2nm_CdSe/filter: input.par, eval.dat)."""
    atyp, xyz = read_conf(os.path.join(GOLD, "cdse22", "conf.par"))
    types = sorted(set(atyp), key=atyp.index)
    # the grid of that run (localPot.cube header); its version used box = n d on odd axes
    g = O.Grid(57, 52, 45, 0.8, 0.8, 0.8, -22.8, -20.8, -18.0, 10.0, box_n=True)
    tabs = [read_pot(os.path.join(GOLD, "cdse22", f"pot{t}.par")) for t in types]
    pot = O.local_pot(g, xyz, np.array([types.index(a) for a in atyp]), tabs)
    targets = _targets(-0.31, -0.24, -0.15, -0.06, 10, 6)
    # the mixed path filters 48 starts: the FP32 recursion's noise (about 1e-4
    # of each filtered state's norm) swamps the directions of the filtered
    # subspace whose overlap eigenvalues lie below ~1e-6 of the largest, so a
    # level that 16 starts carry only in such directions needs more starts
    # (measured on this input: 16 starts match 64 of the 124 levels, 32 match
    # 99, 48 match 107; the FP64 path matches 121 with 16)
    nstart = 48 if precision else 16
    (emin, emax), ev, sg = _run(fbse, cuda, g, pot, targets, 2048, nstart, 1, False, precision=precision)
    # run.dat:140 of the reference run: Emin = -1.13271, Emax = 12.3281.  Both
    # iterations stop at a relative change below 1e-6 per step (energy.c:239,
    # 282), not at the extremum, so the stopping values agree only to ~1e-3.
    assert abs(emin - (-1.13271)) < 3e-3 and abs(emax - 12.3281) < 1e-3 * 12.3281
    ref = np.loadtxt(os.path.join(GOLD, "cdse22", "eval.dat"))
    r, d = _match(ref, ev, sg, 1e-5, MY_SIGMA[precision], 1e-5)
    print(f"\n[cdse22 precision={precision}] ours: {len(ev)} states, {np.sum(sg < 1e-4)} with sigma<1e-4; reference converged "
          f"(sigma<1e-5): {len(r)}; matched within 1e-5: {np.sum(d < 1e-5)}; max |dE| of matched "
          f"{np.max(d[d < 1e-5]) if np.any(d < 1e-5) else np.nan:.2e}")
    assert np.mean(d < 1e-5) >= 0.8


def _so_params(path):
    vals = [float(l.split()[0]) for l in open(path).read().splitlines() if l.strip()]
    return vals[0], vals[1], vals[2]


def _cspbi3_system():
    d = os.path.join(GOLD, "cspbi3")
    atyp, xyz = read_conf(os.path.join(d, "conf.par"))
    types = sorted(set(atyp), key=atyp.index)
    g = O.Grid(44, 44, 44, 0.5, 0.5, 0.5, -11.0, -11.0, -11.0, 20.0)
    tabs = [read_pot(os.path.join(d, f"pot{t}.par")) for t in types]
    pot = O.local_pot(g, xyz, np.array([types.index(a) for a in atyp]), tabs)
    rc = np.sqrt(O.r_nlcut2(g.dx))
    so_tab = O.so_radial(g.dx, rc)
    params = {t: _so_params(os.path.join(d, f"SO_{t}.par")) for t in types}
    cache = {}
    nl_tabs, sgns = [], []
    for a in atyp:
        lam = params[a][1:]
        if lam not in cache:
            cache[lam] = O.nl_radial(g.dx, rc, *lam)
        nl_tabs.append(cache[lam][0])
        sgns.append(cache[lam][1])
    proj = O.nlc_table(g, xyz, np.array([params[a][0] for a in atyp]), so_tab, np.array(nl_tabs), np.array(sgns))
    assert int(proj.npts) == 2325  # n_NL_gridpts in the reference run's run.dat
    return g, pot, proj


@pytest.mark.parametrize("precision", [0, 1])
def test_cspbi3_spinor_so_nl_matches_reference_eval(fbse, cuda, precision):
    """1x1x1 CsPbI3, spinor with spin-orbit and nonlocal projectors, 44^3 at 0.5 bohr
    (filter_mpi/EXAMPLES/1x1x1_CsPbI3/filter: input.par, SO_*.par, reference_output/eval.dat)."""
    d = os.path.join(GOLD, "cspbi3")
    g, pot, proj = _cspbi3_system()
    targets = _targets(-0.50, -0.20, -0.167, -0.10, 10, 6)
    (emin, emax), ev, sg = _run(fbse, cuda, g, pot, targets, 2048, 16, 2, True, so=True, nl=True, proj=proj,
                                precision=precision)
    # run.dat:160 of the reference run: Emin = -0.756627, Emax = 25.2627
    assert abs(emin - (-0.756627)) < 3e-3 and abs(emax - 25.2627) < 1e-3 * 25.2627
    ref = np.loadtxt(os.path.join(d, "eval.dat"))
    r, dd = _match(ref, ev, sg, 1e-6, MY_SIGMA[precision], 1e-5)
    print(f"\n[cspbi3 precision={precision}] ours: {len(ev)} states, {np.sum(sg < 1e-4)} with sigma<1e-4; reference converged: {len(r)};"
          f" matched within 1e-5: {np.sum(dd < 1e-5)}; max |dE| of matched "
          f"{np.max(dd[dd < 1e-5]) if np.any(dd < 1e-5) else np.nan:.2e}")
    assert np.mean(dd < 1e-5) >= 0.8


def test_mixed_subspace_overlap_matches_fp64(fbse, cuda):
    """The mixed path's eigenvectors span the plain FP64 path's: on the same
    starts (CsPbI3, spinor, SO + NL), for every isolated degenerate FP64
    cluster (levels within 1e-6 Ha) converged to sigma_E < 1e-6 whose level the
    mixed run reproduces to 1e-5 Ha with as many pairs (sigma_E <= 1e-2),
    1 - s_min(V_mixed^H V_fp64 dv) <= 1e-6, s_min the smallest singular value
    of the overlap of the two orthonormal cluster bases."""
    g, pot, proj = _cspbi3_system()
    targets = _targets(-0.50, -0.20, -0.167, -0.10, 10, 6)
    out = {}
    for prec in (0, 1):
        _, ev, sg, v = _run(fbse, cuda, g, pot, targets, 2048, 16, 2, True, so=True, nl=True, proj=proj,
                            precision=prec, states=True)
        out[prec] = (ev, sg, v.view(np.complex128))
    (e64, s64, v64), (emx, smx, vmx) = out[0], out[1]
    good64 = np.where(s64 < 1e-6)[0]
    order = good64[np.argsort(e64[good64])]
    worst, nclus = 0.0, 0
    for cl in _clusters(e64[order], 1e-6):
        idx = order[cl]
        e = e64[idx].mean()
        # the cluster must be isolated among the FP64 levels (no partner left out)
        if np.sum(np.abs(e64 - e) < 1e-5) != len(idx):
            continue
        mine = np.where((np.abs(emx - e) < 1e-5) & (smx < 1e-2))[0]
        if len(mine) != len(idx):
            continue
        ov = vmx[mine].conj() @ v64[idx].T * g.dv
        smin = np.linalg.svd(ov, compute_uv=False).min()
        worst = max(worst, 1.0 - smin)
        nclus += 1
    print(f"\n[cspbi3 mixed vs fp64] {nclus} converged clusters compared, max 1 - s_min = {worst:.2e}")
    assert nclus >= 10 and worst <= 1e-6


def _clusters(e, tol=1e-6):
    """Groups of consecutive energies closer than tol (degenerate excitons)."""
    out, cur = [], [0]
    for i in range(1, len(e)):
        if e[i] - e[i - 1] < tol:
            cur.append(i)
        else:
            out.append(cur)
            cur = [i]
    out.append(cur)
    return out


def test_cspbi3_bse_matches_reference_exciton(fbse, cuda):
    """BSE on the filtered 1x1x1 CsPbI3 spinors against the reference's own run
    (bse_cplx/EXAMPLES/1x1x1_CsPbI3/bse: input.par, reference_output/exciton.dat
    and OS.dat).  That run's basis (OS0.dat) was 8 holes and 8 electrons: the
    top 8 converged states below fermiEnergy = -0.19 and the lowest 8 above
    (get_qp_basis_indices, bse_cplx/basis.c:7-254).  Its 8 holes hold only 2 of
    the 4 states of the exactly degenerate level at -0.2873 Ha, an arbitrary
    2-dimensional subspace of the 4 that the reference's own diagonalisation
    picked.  Excitons that do not feel that choice must match to 1e-6 Ha; for
    all excitons the reference energy must lie in the range spanned by random
    choices of that subspace."""
    import torch
    d = os.path.join(GOLD, "cspbi3")
    atyp, xyz = read_conf(os.path.join(d, "conf.par"))
    types = sorted(set(atyp), key=atyp.index)
    g = O.Grid(44, 44, 44, 0.5, 0.5, 0.5, -11.0, -11.0, -11.0, 20.0)
    tabs = [read_pot(os.path.join(d, f"pot{t}.par")) for t in types]
    pot = O.local_pot(g, xyz, np.array([types.index(a) for a in atyp]), tabs)
    rc = np.sqrt(O.r_nlcut2(g.dx))
    so_tab = O.so_radial(g.dx, rc)
    params = {t: _so_params(os.path.join(d, f"SO_{t}.par")) for t in types}
    nl_tabs, sgns = [], []
    for a in atyp:
        t_, s_ = O.nl_radial(g.dx, rc, *params[a][1:])
        nl_tabs.append(t_)
        sgns.append(s_)
    proj = O.nlc_table(g, xyz, np.array([params[a][0] for a in atyp]), so_tab, np.array(nl_tabs), np.array(sgns))
    ctx = fbse.Context(g, pot, nspin=2, is_complex=True, so=True, nl=True, proj=proj, precision=0)
    e0, e1, _ = ctx.energy_range()
    emin = e0 - 0.2 * abs(e0)
    de = e1 * 1.2 - emin
    zn, _ = fbse.samp_points(2048)
    targets = _targets(-0.30, -0.24, -0.11, 0.01, 8, 8)  # around the gap: the basis states of that run
    an = fbse.newton_coeff(zn, targets, emin, de, O.filter_dt(2048, de))
    starts, _, _ = fbse.init_filter_states(16, g.ngrid, 2, True, g.dv, -31415)
    filt = ctx.newton_filter(zn, an, emin, de, torch.tensor(starts, device=cuda))
    psitot = filt.reshape(16 * len(targets), -1)
    nk, ev, sg = ctx.ortho_diag_sigma(psitot)
    psi = psitot[:nk].view(torch.complex128)
    par = dict(l.split("=") for l in open(os.path.join(d, "bse_input.par")).read().splitlines() if "=" in l)
    par = {k.strip(): float(v) for k, v in par.items()}
    fermi, eps, cut = par["fermiEnergy"], par["epsX"], par["sigmaECut"]
    conv = np.where(sg < cut)[0]
    holes = [i for i in conv if ev[i] < fermi][-8:]
    elecs = [i for i in conv if ev[i] > fermi][:8]
    assert len(holes) == 8 and len(elecs) == 8
    quart = [i for i in range(nk) if abs(ev[i] - ev[holes[0]]) < 1e-8]
    assert len(quart) == 4 and holes[:2] == quart[2:]
    bctx = fbse.Context(g, np.zeros(g.ngrid), nspin=2, is_complex=True, precision=0)
    gx, gy, gz = O.bse_axes(g)
    bare, scr = bctx.bse_potentials(gx, gy, gz, g.xmin, g.ymin, g.zmin, (eps, par["epsY"], par["epsZ"]))
    rest = holes[2:]
    evq = np.concatenate([[ev[quart[0]]] * 2, ev[rest], ev[elecs]])
    rng = np.random.default_rng(0)
    samples = []
    for smp in range(16):
        if smp == 0:
            Q = psi[holes[:2]]
        else:
            U, _ = np.linalg.qr(rng.normal(size=(4, 4)) + 1j * rng.normal(size=(4, 4)))
            Q = torch.tensor(U.T[:2].copy(), device=cuda) @ psi[quart]
        qp = torch.cat([Q, psi[rest], psi[elecs]]).contiguous()
        Kd, Kx = bctx.bse_kernel(qp, 8, 8, 8, bare, scr)
        e, C, hh, dd, xx, h0 = bctx.bse_solve(evq, 8, 8, 8, Kd, Kx)
        mu = bctx.bse_dipoles(qp, gx, gy, gz, 8, 8, 8)
        mx = bctx.bse_optical(C, mu, 8, 8)
        samples.append((e, dd, xx, h0, np.sum(np.abs(mx) ** 2, axis=1)))
        if smp == 0:
            # magnetic dipoles and rotational strengths (calc_mag_dipole,
            # calc_rotational_strength, calc_optical_exc) of the same basis
            mm = bctx.bse_mag_dipoles(qp, gx, gy, gz, 8, 8, 8)
            mmx = bctx.bse_optical(C, mm, 8, 8)
            mag0 = (mu, mm, mx, mmx)
    E = np.array([s[0] for s in samples])
    ref = np.loadtxt(os.path.join(d, "exciton.dat"))
    osr = np.loadtxt(os.path.join(d, "OS.dat"))
    spread = E.max(0) - E.min(0)
    fixed = spread < 1e-7
    print(f"\n[cspbi3 bse] {np.sum(fixed)} of 64 excitons independent of the degenerate subspace; max |dE| there "
          f"{np.max(np.abs(E[0] - ref[:, 1])[fixed]):.2e}; max spread elsewhere {spread.max():.2e}")
    assert np.sum(fixed) >= 32
    assert np.all(np.abs(E[0] - ref[:, 1])[fixed] < 1e-6)
    # random subspaces sample the admissible range from inside: allow half the
    # sampled spread beyond it on either side
    margin = 0.5 * spread + 1e-6
    assert np.all((ref[:, 1] >= E.min(0) - margin) & (ref[:, 1] <= E.max(0) + margin))
    # <K^d>, <K^x>, <h0> and |mu|^2 summed over degenerate clusters (invariant within a cluster)
    e0s, d0, x0, h00, m0 = samples[0]
    for cl in _clusters(ref[:, 1]):
        if not np.all(fixed[cl]):
            continue
        assert abs(np.sum(d0[cl]) - np.sum(ref[cl, 3])) < 1e-6
        assert abs(np.sum(x0[cl]) - np.sum(ref[cl, 4])) < 1e-6
        assert abs(np.sum(h00[cl]) - np.sum(ref[cl, 5])) < 1e-6
        assert abs(np.sum(m0[cl]) - np.sum(osr[cl, 1] ** 2)) < 1e-5 * max(1.0, np.sum(osr[cl, 1] ** 2))
    # M.dat / rs.dat: |m_j|^2 and Im(mu_j . conj m_j) summed over the same clusters
    mu, mm, mx, mmx = mag0
    Mr = np.loadtxt(os.path.join(d, "M.dat"))
    rsr = np.loadtxt(os.path.join(d, "rs.dat"))
    m2 = np.sum(np.abs(mmx) ** 2, axis=1)
    rsx = np.sum(np.imag(mx * np.conj(mmx)), axis=1)
    worst_m = worst_rs = 0.0
    for cl in _clusters(ref[:, 1]):
        if not np.all(fixed[cl]):
            continue
        worst_m = max(worst_m, abs(np.sum(m2[cl]) - np.sum(Mr[cl, 1] ** 2)))
        worst_rs = max(worst_rs, abs(np.sum(rsx[cl]) - np.sum(rsr[cl, 2])))
    # pair level (M0.dat, rs0.dat): sums over Kramers-degenerate hole and electron
    # levels, leaving out the two holes of the partly included quartet
    M0r = np.loadtxt(os.path.join(d, "M0.dat"))
    rs0r = np.loadtxt(os.path.join(d, "rs0.dat"))
    lv = lambda idx: [[idx[k] for k in cl] for cl in _clusters(evq[idx])]
    holes_lv, elec_lv = lv(list(range(2, 8))), lv(list(range(8, 16)))
    worst_m0 = worst_rs0 = 0.0
    scale_m0 = np.max(M0r[:, 2] ** 2)
    # the files list (i, a) in different orders (M0.dat a-major, rs0.dat i-major)
    row_m0 = {(int(r[0]), int(r[1])): k for k, r in enumerate(M0r)}
    row_rs0 = {(int(r[0]), int(r[1])): k for k, r in enumerate(rs0r)}
    for H in holes_lv:
        for A in elec_lv:
            pairs = [(i, a) for i in H for a in A]
            mine_rows = [i * 8 + (a - 8) for i, a in pairs]  # this library: i * n_e + (a - lumo)
            mine = np.sum(np.abs(mm[mine_rows]) ** 2)
            ref_m = np.sum(M0r[[row_m0[p] for p in pairs], 2] ** 2)
            worst_m0 = max(worst_m0, abs(mine - ref_m) / scale_m0)
            mine_rs = np.sum(np.imag(np.sum(mu[mine_rows] * np.conj(mm[mine_rows]), axis=1)))
            ref_rs = np.sum(rs0r[[row_rs0[p] for p in pairs], 3])
            # the cube is centrosymmetric: rotational strengths vanish up to the
            # grid's asymmetry and the states' convergence, so they can only
            # agree on the scale |mu| |m| of the block
            rs_scale = np.sqrt(np.sum(np.abs(mu[mine_rows]) ** 2) * mine)
            worst_rs0 = max(worst_rs0, abs(mine_rs - ref_rs) / rs_scale)
    print(f"[cspbi3 bse] magnetic: exciton |m|^2 max dev {worst_m:.2e} (max {Mr[:, 1].max() ** 2:.2e}), rs {worst_rs:.2e}; "
          f"pairs |m|^2 rel {worst_m0:.2e}, rs0 rel to |mu||m| {worst_rs0:.2e}")
    assert worst_m0 < 1e-4 and worst_rs0 < 3e-3
    assert worst_m < 1e-4 * Mr[:, 1].max() ** 2
    assert worst_rs < 1e-4 * np.sqrt(np.max(np.sum(np.abs(mx) ** 2, axis=1)) * Mr[:, 1].max() ** 2)
