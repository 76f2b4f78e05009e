"""MLP-3c in the assembly: routing, the error gate and what the trained
network gains.  The reference is the FP64 oracle (the table path equals it
to 1e-10 eV); tolerances are stated in Hartree as the surrogate's contract
is (1 Ha = P_eq2 / P_abohr eV)."""
import numpy as np
import pytest

from conftest import symmetric_denmat, workload
from oracle import oracle as orc

pytestmark = pytest.mark.gpu

P_HARTREE = 14.39975 / 0.529177  # eV
P_EQ2 = 14.39975


@pytest.fixture(scope="module")
def mlp_sys(fdata_root):
    import fbgpu
    path, nZ, st = workload("sic_small", fdata_root)
    fd = orc.Fdata(path, nZ)
    s = orc.System(fd, st.ratom, st.imass, st.lattice).neighbors()
    blocks = s.assemble()
    norb = np.array([fd.norb(int(k)) for k in st.imass])
    rho, cape = symmetric_denmat(s, norb, 21)
    fref = s.dassemble(rho, cape)
    ctx = fbgpu.Context(0)
    ctx.read_Fdata(path, nZ)
    ctx.set_structure(st.ratom, st.imass, st.lattice)
    ctx.driver_neighbors()
    ctx.mlp_init(seed=5)
    untrained = ctx.mlp_validate(samples_per_bin=8, seed=1)
    untrained_bins = ctx.mlp_bin_errors()
    hist = ctx.mlp_train(nsamples=1 << 18, epochs=8, batch=2048, lr=3e-3, seed=9)
    trained = ctx.mlp_validate(samples_per_bin=16, seed=2)
    yield dict(ctx=ctx, st=st, blocks=blocks, rho=rho, cape=cape, fref=fref, hist=hist,
               untrained=untrained, untrained_bins=untrained_bins, trained=trained, s=s)
    ctx.close()


def _run(ctx, rho, cape):
    ctx.assemble()
    out = {k: ctx.blocks(k) for k in ("S", "T", "vna", "vnao")}
    ctx.set_denmat(rho, cape)
    ctx.Dassemble()
    out.update({k: ctx.forces(k) for k in ("ftot", "f3naa", "f3nab", "f3nac")})
    return out


def _nmax(s):
    return int(np.bincount(s.cneigh[:s.ntrip] + s.pair_off[s.ci_j[:s.ntrip]]).max())


def test_training_converges(mlp_sys):
    h = mlp_sys["hist"]
    assert np.all(np.isfinite(h)) and h[-1] < 0.2 * h[0], h
    assert mlp_sys["trained"] < mlp_sys["untrained"]


def test_off_is_the_table_path(mlp_sys):
    import fbgpu
    ctx = mlp_sys["ctx"]
    ctx.mlp_set_mode(fbgpu.FB_MLP_OFF)
    assert ctx.mlp_routed()[0] == 0
    got = _run(ctx, mlp_sys["rho"], mlp_sys["cape"])
    for key, ref in zip(("S", "T", "vna", "vnao"), mlp_sys["blocks"]):
        assert np.abs(got[key] - ref).max() <= 1e-10


def test_all_mlp_errors_bounded(mlp_sys):
    """Every triplet through the network: 2c blocks untouched, the vna error
    within the worst-case bound of the validated per-triplet error."""
    import fbgpu
    ctx, s = mlp_sys["ctx"], mlp_sys["s"]
    ctx.mlp_set_mode(fbgpu.FB_MLP_ALL)
    n_mlp, n_all = ctx.mlp_routed()
    assert n_mlp == n_all == s.ntrip
    got = _run(ctx, mlp_sys["rho"], mlp_sys["cape"])
    S0, T0, vb0, vbo0 = mlp_sys["blocks"]
    assert np.abs(got["S"] - S0).max() <= 1e-10
    assert np.abs(got["T"] - T0).max() <= 1e-10
    assert np.abs(got["vnao"] - vbo0).max() <= 1e-10
    err = np.abs(got["vna"] - vb0).max()
    bound = 2.0 * P_EQ2 * 3.0 * _nmax(s) * mlp_sys["trained"]   # sampled maximum: factor 2 margin
    assert 0.0 < err <= bound, (err, bound)
    assert np.all(np.isfinite(got["ftot"]))
    ctx.mlp_set_mode(fbgpu.FB_MLP_OFF)


@pytest.mark.parametrize("quantile", [0.25, 0.75])
def test_gate_holds_tolerance(mlp_sys, quantile):
    """A tolerance that approves part of the bins: the measured |dH| (Ha)
    stays within it and the 2c blocks are untouched."""
    import fbgpu
    ctx, s = mlp_sys["ctx"], mlp_sys["s"]
    errs = ctx.mlp_bin_errors()
    errs = errs[errs > 0]
    tau_target = float(np.quantile(errs, quantile))
    tol_ha = tau_target * P_EQ2 * 3.0 * _nmax(s) / P_HARTREE
    tau, cov = ctx.mlp_gate(tol_ha)
    assert abs(tau - tau_target) <= 1e-6 * tau_target
    got = _run(ctx, mlp_sys["rho"], mlp_sys["cape"])
    dH = np.abs(got["vna"] - mlp_sys["blocks"][2]).max() / P_HARTREE
    assert dH <= tol_ha, (dH, tol_ha, cov)
    assert ctx.mlp_routed()[0] == round(cov * s.ntrip)
    ctx.mlp_set_mode(fbgpu.FB_MLP_OFF)


def test_tiny_tolerance_falls_back(mlp_sys):
    """At 1e-12 Ha no bin qualifies: the gated path is the table path."""
    import fbgpu
    ctx = mlp_sys["ctx"]
    tau, cov = ctx.mlp_gate(1e-12)
    assert cov == 0.0 and ctx.mlp_routed()[0] == 0
    got = _run(ctx, mlp_sys["rho"], mlp_sys["cape"])
    assert np.abs(got["vna"] - mlp_sys["blocks"][2]).max() <= 1e-10
    ctx.mlp_set_mode(fbgpu.FB_MLP_OFF)


def test_trained_network_gains(mlp_sys):
    """What training buys: at the tolerance where the trained network takes
    half of the bins, the untrained one takes (almost) none."""
    errs = mlp_sys["ctx"].mlp_bin_errors()
    ue = mlp_sys["untrained_bins"]
    used = errs > 0
    tau = float(np.median(errs[used]))
    trained_share = float(np.mean(errs[used] <= tau))
    untrained_share = float(np.mean(ue[used] <= tau))
    assert trained_share >= 0.5
    assert untrained_share <= 0.05 * trained_share, (trained_share, untrained_share)


def _legendre(c):
    c2 = c * c
    p = np.stack([np.ones_like(c), c, 0.5 * (3 * c2 - 1), 0.5 * c * (5 * c2 - 3), 0.125 * (3 - c2 * (30 - 35 * c2))], -1)
    return p


def test_eval_points_match_oracle(mlp_sys):
    """The assembly's network evaluation (values and forward-mode tangents)
    against the CPU oracle network: values with the same BF16 roundings,
    derivatives against central differences of the unrounded network."""
    from fbgpu import synth
    from oracle import mlp_oracle as mo
    ctx = mlp_sys["ctx"]
    sp = synth.species_for("sic4096")
    rng = np.random.default_rng(4)
    n = 96
    trip = rng.integers(0, 8, n)
    xmax = np.array([sp[t % 2].rcA + max(sp[t // 4].rcA, sp[(t // 2) % 2].rcA) for t in trip])
    ymax = np.array([sp[t // 4].rcA + sp[(t // 2) % 2].rcA for t in trip])
    x = rng.uniform(0.05, 0.95, n) * xmax
    y = rng.uniform(0.05, 0.95, n) * ymax
    c = rng.uniform(-0.95, 0.95, n)
    got = ctx.mlp_eval_points(np.stack([x, y, c], 1), trip)
    P = mo.unpack(ctx.mlp_params(), ctx.mlp_offsets)
    scale = ctx.mlp_scales()

    def combined(xx, yy, cc, exact):
        feat = np.stack([2 * xx / xmax - 1, 2 * yy / ymax - 1, cc], 1)
        out, _ = mo.forward(P, feat, trip, exact=exact)
        v = out[:, :50].reshape(n, 5, 10) * scale[trip, :50].reshape(n, 5, 10)
        return np.einsum("nt,nte->ne", _legendre(cc), v)

    ref = combined(x, y, c, exact=False)
    vs = np.abs(ref).max()
    assert np.abs(got[:, 0] - ref).max() <= 2e-2 * vs
    h = 1e-4
    dref = [(combined(x, y, c + h, True) - combined(x, y, c - h, True)) / (2 * h),
            (combined(x + h, y, c, True) - combined(x - h, y, c, True)) / (2 * h),
            (combined(x, y + h, c, True) - combined(x, y - h, c, True)) / (2 * h)]
    for k, d in enumerate(dref):
        ds = np.abs(d).max()
        err = np.abs(got[:, k + 1] - d)
        assert err.max() <= 5e-2 * ds, (k, err.max(), ds)
        assert err.mean() <= 1e-2 * ds, (k, err.mean(), ds)


def test_mlp_forces_track_table_forces(mlp_sys):
    """All triplets through the network: the three-center forces stay close
    to the table path's (a wiring check; their error is the network's
    derivative error)."""
    import fbgpu
    ctx = mlp_sys["ctx"]
    ctx.mlp_set_mode(fbgpu.FB_MLP_ALL)
    got = _run(ctx, mlp_sys["rho"], mlp_sys["cape"])
    ctx.mlp_set_mode(fbgpu.FB_MLP_OFF)
    f = mlp_sys["fref"]
    f3 = got["f3naa"] + got["f3nab"] + got["f3nac"]
    f3ref = f["f3naa"] + f["f3nab"] + f["f3nac"]
    rel = np.linalg.norm(f3 - f3ref) / np.linalg.norm(f3ref)
    assert rel < 0.3, rel


def test_tcgen05_engine_matches_mma(mlp_sys):
    """The tcgen05 evaluation (TMEM accumulators) against the mma.sync one:
    the same network and roundings, FP32 sums in another order."""
    import fbgpu
    from fbgpu import synth
    ctx = mlp_sys["ctx"]
    sp = synth.species_for("sic4096")
    rng = np.random.default_rng(12)
    n = 300   # not a multiple of 128: a partial tile
    trip = rng.integers(0, 8, n)
    xmax = np.array([sp[t % 2].rcA + max(sp[t // 4].rcA, sp[(t // 2) % 2].rcA) for t in trip])
    ymax = np.array([sp[t // 4].rcA + sp[(t // 2) % 2].rcA for t in trip])
    pts = np.stack([rng.uniform(0.02, 0.98, n) * xmax, rng.uniform(0.02, 0.98, n) * ymax,
                    rng.uniform(-1, 1, n)], 1)
    ctx.mlp_set_engine(fbgpu.FB_MLP_ENGINE_MMA)
    ref = ctx.mlp_eval_points(pts, trip)
    ref0 = ctx.mlp_eval_points(pts, trip, derivs=False)
    ctx.mlp_set_engine(fbgpu.FB_MLP_ENGINE_TC)
    got = ctx.mlp_eval_points(pts, trip)
    got0 = ctx.mlp_eval_points(pts, trip, derivs=False)
    ctx.mlp_set_engine(fbgpu.FB_MLP_ENGINE_MMA)
    for k in range(4):
        s = np.abs(ref[:, k]).max()
        assert np.abs(got[:, k] - ref[:, k]).max() <= 2e-2 * s, k
        assert np.abs(got[:, k] - ref[:, k]).mean() <= 2e-3 * s, k
    assert np.abs(got0 - ref0).max() <= 2e-2 * np.abs(ref0).max()
    assert np.abs(got0 - got[:, 0]).max() <= 2e-2 * np.abs(ref0).max()


def test_tcgen05_engine_in_the_assembly(mlp_sys):
    import fbgpu
    ctx = mlp_sys["ctx"]
    ctx.mlp_set_mode(fbgpu.FB_MLP_ALL)
    ctx.mlp_set_engine(fbgpu.FB_MLP_ENGINE_MMA)
    a = _run(ctx, mlp_sys["rho"], mlp_sys["cape"])
    ctx.mlp_set_engine(fbgpu.FB_MLP_ENGINE_TC)
    b = _run(ctx, mlp_sys["rho"], mlp_sys["cape"])
    ctx.mlp_set_engine(fbgpu.FB_MLP_ENGINE_MMA)
    ctx.mlp_set_mode(fbgpu.FB_MLP_OFF)
    v0 = mlp_sys["blocks"][2]
    assert np.abs(b["vna"] - a["vna"]).max() <= 0.05 * np.abs(a["vna"] - v0).max() + 1e-9
    assert np.linalg.norm(b["ftot"] - a["ftot"]) <= 0.05 * np.linalg.norm(a["ftot"])
