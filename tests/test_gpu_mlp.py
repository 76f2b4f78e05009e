"""MLP-3c surrogate on the GPU: training samples against the oracle's table
interpolation, the library's forward pass and gradient against the CPU
oracle MLP (same BF16 roundings), and training lowering the loss."""
import numpy as np
import pytest

from fbgpu import synth
from oracle import mlp_oracle as mo
from oracle import oracle as orc

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def mlp_ctx(fdata_root):
    import fbgpu
    path = synth.fdata_dir_for("sic4096", root=fdata_root)
    ctx = fbgpu.Context(0)
    ctx.read_Fdata(path, [14, 6])
    ctx.mlp_init(seed=11)
    yield ctx, path
    ctx.close()


def _legendre(c):
    return np.array([1.0, c, 0.5 * (3 * c * c - 1), 0.5 * c * (5 * c * c - 3),
                     0.125 * (3 - c * c * (30 - 35 * c * c))])


def test_samples_match_table_interpolation(mlp_ctx):
    """sum_theta P_theta(cos) * target * scale is getMEs_Fdata_3c (bcna)."""
    ctx, path = mlp_ctx
    sp = synth.species_for("sic4096")
    nsp = len(sp)
    fd = orc.Fdata(path, [14, 6])
    f, t, y = ctx.mlp_samples(256, seed=5)
    scale = ctx.mlp_scales()
    for r in range(0, 256, 7):
        tr = int(t[r])
        a, b, k = tr // (nsp * nsp), (tr // nsp) % nsp, tr % nsp
        A, B, K = sp[a], sp[b], sp[k]
        u, v, c = (float(f[r, 0]) + 1) / 2, (float(f[r, 1]) + 1) / 2, float(f[r, 2])
        xmax = K.rcA + max(A.rcA, B.rcA)
        ymax = A.rcA + B.rcA
        mu, nu, mv = synth.make_munu_3c(A.lssh, B.lssh)
        na, nb = sum(2 * l + 1 for l in A.lssh), sum(2 * l + 1 for l in B.lssh)
        ref = orc.getMEs_3c(fd, a + 1, b + 1, k + 1, u * xmax, v * ymax, c, na, nb)
        pl = _legendre(c)
        sint = np.sqrt(max(1e-5, 1 - c * c))
        for e in range(len(mu)):
            val = sum(pl[th] * y[r, th * 10 + e] * scale[tr, th * 10 + e] for th in range(5))
            if mv[e] == 1:
                val *= sint
            assert abs(val - ref[mu[e] - 1, nu[e] - 1]) <= 2e-6 * max(1.0, abs(ref[mu[e] - 1, nu[e] - 1])), (r, e)


def _nme(ctx):
    """bcna matrix elements of every species triple"""
    sp = synth.species_for("sic4096")
    out = []
    for a in sp:
        for b in sp:
            for _k in sp:
                out.append(len(synth.make_munu_3c(a.lssh, b.lssh)[0]))
    return np.array(out)


BF16_ULP = 2.0 ** -8  # relative spacing of BF16 (8 significand bits)


def test_forward_matches_oracle(mlp_ctx):
    """Per output column.  The oracle applies the same BF16 roundings of
    weights and layer inputs, so the two differ only by FP32 accumulation
    order and by the layer inputs whose FP32 values sit on a BF16 rounding
    boundary (a one-ulp flip, 2^-8 relative).  Four rounded layer inputs
    bound a column's largest error by 4 ulp of the column's scale, and its
    RMS error by one ulp of its RMS: a wrong layout or scale of any one
    column breaks both."""
    ctx, _ = mlp_ctx
    f, t, y = ctx.mlp_samples(512, seed=6)
    out = ctx.mlp_forward(f, t)
    P = mo.unpack(ctx.mlp_params(), ctx.mlp_offsets)
    ref, _ = mo.forward(P, f.astype(np.float64), t)
    floor = 1e-6 * np.abs(ref).max()
    col_err = np.abs(out - ref).max(axis=0)
    col_scale = np.abs(ref).max(axis=0)
    bad = np.nonzero(col_err > 4 * BF16_ULP * col_scale + floor)[0]
    assert len(bad) == 0, (bad, col_err[bad], col_scale[bad])
    col_rms_err = np.sqrt(np.mean((out - ref) ** 2, axis=0))
    col_rms = np.sqrt(np.mean(ref ** 2, axis=0))
    bad = np.nonzero(col_rms_err > BF16_ULP * col_rms + floor)[0]
    assert len(bad) == 0, (bad, col_rms_err[bad], col_rms[bad])


def test_gradient_matches_oracle(mlp_ctx):
    ctx, _ = mlp_ctx
    f, t, y = ctx.mlp_samples(256, seed=8)
    loss, g = ctx.mlp_grad(f, t, y)
    P = mo.unpack(ctx.mlp_params(), ctx.mlp_offsets)
    lref, gref = mo.loss_and_grad(P, f.astype(np.float64), t, y.astype(np.float64), _nme(ctx))
    assert abs(loss - lref) <= 1e-3 * abs(lref)
    G = mo.unpack(g, ctx.mlp_offsets)
    for k in ("emb", "W1", "b1", "W2", "b2", "W3", "b3", "W4", "b4"):
        num = np.linalg.norm(G[k] - gref[k])
        den = np.linalg.norm(gref[k])
        assert num <= 2e-2 * den + 1e-12, (k, num / max(den, 1e-300))


def test_training_lowers_loss(mlp_ctx):
    ctx, _ = mlp_ctx
    f, t, y = ctx.mlp_samples(4096, seed=99)
    l0, _ = ctx.mlp_grad(f, t, y)
    hist = ctx.mlp_train(nsamples=1 << 16, epochs=4, batch=1024, lr=2e-3, seed=3)
    l1, _ = ctx.mlp_grad(f, t, y)
    assert np.all(np.isfinite(hist))
    assert hist[-1] < hist[0]
    assert l1 < 0.5 * l0, (l0, l1)
