"""The learned initial guess: gradients of the GPU training kernels against a
CPU float64 autograd restatement of the same network, and the gain of the
trained network over the zero guess on held-out solves."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

LAYERS = [(5, 16), (16, 16), (16, 32), (32, 32), (32, 64), (64, 64), (64, 64), (64, 64),
          (128, 64), (64, 64), (96, 32), (32, 32), (48, 16), (16, 16)]


def unpack(params):
    """Per-layer (W[27][cout][cin], b[cout]) and the head (w[16], b)."""
    out, o = [], 0
    for cin, cout in LAYERS:
        w = params[o:o + 27 * cout * cin].reshape(27, cout, cin)
        o += 27 * cout * cin
        b = params[o:o + cout]
        o += cout
        out.append((w, b))
    head = params[o:o + 17]
    assert o + 17 == params.size
    return out, head


def interp_matrix(nf, nc, periodic):
    """Cell-centred linear interpolation from nc coarse to nf fine cells
    (weights 3/4, 1/4 on the two nearest coarse cells; clamped or periodic)."""
    P = np.zeros((nf, nc))
    for x in range(nf):
        c = x >> 1
        c0, c1, w0, w1 = (c, c + 1, 0.75, 0.25) if x & 1 else (c - 1, c, 0.25, 0.75)
        if periodic:
            c0, c1 = c0 % nc, c1 % nc
        else:
            c0, c1 = max(c0, 0), min(c1, nc - 1)
        P[x, c0] += w0
        P[x, c1] += w1
    return P


def torch_reference(params, feat, target, mask, X, Y, Z):
    """Loss and parameter gradients in float64 on the CPU (storage rounded to
    BF16 where the GPU stores BF16: weights, inputs, activations).  The inputs
    are averaged over 2x2x2 cells, the network runs on that half-resolution
    grid and its output is interpolated back to the grid (trilinear); the loss
    is taken on the full grid."""
    torch = pytest.importorskip("torch")
    F = torch.nn.functional

    class RoundBF16(torch.autograd.Function):
        @staticmethod
        def forward(ctx, x):
            return x.to(torch.bfloat16).to(torch.float64)

        @staticmethod
        def backward(ctx, g):
            return g

    rb = RoundBF16.apply
    layers, head = unpack(params)
    P = []
    for w, b in layers:
        P.append(torch.tensor(w, dtype=torch.float64, requires_grad=True))
        P.append(torch.tensor(b, dtype=torch.float64, requires_grad=True))
    hw = torch.tensor(head, dtype=torch.float64, requires_grad=True)

    def conv(x, l, act=True):
        cin, cout = LAYERS[l]
        w = rb(P[2 * l]).reshape(3, 3, 3, cout, cin).permute(3, 4, 0, 1, 2)
        xp = F.pad(x, (1, 1, 0, 0, 1, 1))                       # zero in r (W) and theta (D)
        xp = torch.cat([xp[:, :, :, -1:, :], xp, xp[:, :, :, :1, :]], dim=3)  # periodic phi (H)
        y = F.conv3d(xp, w, P[2 * l + 1])
        if act:
            y = F.leaky_relu(y, 0.1)
        return rb(y)

    def pool(x):
        Zc, Yc, Xc = [(s + 1) // 2 for s in x.shape[2:]]
        pad = (0, 2 * Xc - x.shape[4], 0, 2 * Yc - x.shape[3], 0, 2 * Zc - x.shape[2])
        s = F.avg_pool3d(F.pad(x, pad), 2, divisor_override=1)
        ones = torch.ones((1, 1) + tuple(x.shape[2:]), dtype=torch.float64)
        cnt = F.avg_pool3d(F.pad(ones, pad), 2, divisor_override=1)
        return rb(s / cnt)

    def up(x, like):
        y = x.repeat_interleave(2, 2).repeat_interleave(2, 3).repeat_interleave(2, 4)
        return y[:, :, :like.shape[2], :like.shape[3], :like.shape[4]]

    f = torch.tensor(feat.reshape(Z, Y, X, 5), dtype=torch.float64).permute(3, 0, 1, 2)[None]
    f = pool(f)                     # averaged over 2x2x2 cells, then BF16: the network runs at half resolution
    s0 = conv(conv(f, 0), 1)
    s1 = conv(conv(pool(s0), 2), 3)
    s2 = conv(conv(pool(s1), 4), 5)
    b3 = conv(conv(pool(s2), 6), 7)
    d2 = conv(conv(torch.cat([up(b3, s2), s2], 1), 8), 9)
    d1 = conv(conv(torch.cat([up(d2, s1), s1], 1), 10), 11)
    d0 = conv(conv(torch.cat([up(d1, s0), s0], 1), 12), 13)
    half = (d0[0] * hw[:16].reshape(16, 1, 1, 1)).sum(0) + hw[16]
    Pz, Py, Px = (torch.tensor(interp_matrix(n, (n + 1) // 2, per)) for n, per in ((Z, False), (Y, True), (X, False)))
    pred = torch.einsum("za,yb,xc,abc->zyx", Pz, Py, Px, half)
    t = torch.tensor(target.reshape(Z, Y, X), dtype=torch.float64)
    m = torch.tensor(mask.reshape(Z, Y, X).astype(np.float64))
    loss = ((pred - t) ** 2 * m).sum() / m.sum()
    loss.backward()
    grads = []
    for l in range(len(LAYERS)):
        grads.append(P[2 * l].grad.numpy().ravel())
        grads.append(P[2 * l + 1].grad.numpy().ravel())
    grads.append(hw.grad.numpy())
    return float(loss.detach()), np.concatenate(grads), pred.detach().numpy().ravel()


def test_gradients_match_cpu_reference():
    from ttcode_gb300 import guess
    from ttcode_gb300.fld import FLD
    from ttcode_gb300.grid import gitter
    from ttcode_gb300.synthetic import default_params
    X, Y, Z = 12, 8, 10
    f = FLD(gitter(X, Y, Z, 7.0e9, 7.7e9), default_params())
    guess.init(f, seed=3)
    blob = guess.save_weights(f)
    params = np.frombuffer(blob[16:], dtype=np.float32).astype(np.float64)
    rng = np.random.default_rng(0)
    V = X * Y * Z
    feat = rng.uniform(-1, 1, (V, 5)).astype(np.float32)
    target = rng.normal(0, 1, V).astype(np.float32)
    mask = (rng.random(V) < 0.8).astype(np.uint8)
    n = guess.num_params()
    g_gpu = np.zeros(n, dtype=np.float32)
    loss = ctypes.c_double()
    rc = f.L.ttfld_guess_gradients(f.h, feat.ctypes.data, target.ctypes.data, mask.ctypes.data,
                                   ctypes.byref(loss), g_gpu.ctypes.data)
    assert rc == 0
    pred_gpu = np.zeros(V, dtype=np.float32)
    assert f.L.ttfld_guess_predict(f.h, feat.ctypes.data, pred_gpu.ctypes.data) == 0
    l_ref, g_ref, pred_ref = torch_reference(params, feat, target, mask, X, Y, Z)
    assert abs(loss.value - l_ref) <= 2e-2 * l_ref
    assert np.linalg.norm(pred_gpu - pred_ref) <= 2e-2 * np.linalg.norm(pred_ref)
    layers, _ = unpack(np.arange(n, dtype=np.float64))
    o = 0
    for l, (cin, cout) in enumerate(LAYERS):
        for size in (27 * cout * cin, cout):
            a, b = g_gpu[o:o + size].astype(np.float64), g_ref[o:o + size]
            err = np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30)
            assert err < 6e-2, (l, size, err)
            o += size
    a, b = g_gpu[o:], g_ref[o:]
    assert np.linalg.norm(a - b) <= 3e-2 * np.linalg.norm(b)


def test_trained_guess_saves_sweeps():
    """Train on 16 solver-generated pairs (random irradiation, dt in [50,500] s)
    on the 100x256x128 shell; on 3 held-out cases the learned guess passes
    the fallback test (no fallback) and needs fewer sweeps to
    ||b-Ax||_1/||b||_1 <= 1e-10 than the zero guess, for the same answer."""
    from ttcode_gb300 import guess
    from ttcode_gb300.fld import start_run
    from ttcode_gb300.synthetic import make_shell
    sh = make_shell(100, 256, 128, seed=2, delt=100.0)
    f = start_run(sh)
    guess.init(f, seed=1, capacity=16)
    assert guess.capture_pairs(f, sh, guess.random_cases(16, seed=10)) == 16
    losses = [guess.train(f, epochs=1, lr=5e-4, seed=e) for e in range(12)]
    assert losses[-1] < 0.05 * losses[0]
    for case in guess.random_cases(3, seed=99):
        z = guess.sweeps_with(f, sh, case, "zero")
        ez = f.download("ER")
        l = guess.sweeps_with(f, sh, case, "learned")
        el = f.download("ER")
        assert l[2] == 0                      # the guess was kept
        assert l[0] < 0.9 * z[0], (l, z)      # at least 10% fewer sweeps
        assert np.linalg.norm(el - ez) <= 1e-9 * np.linalg.norm(ez)


def test_tcgen05_and_mma_sync_convolutions_agree():
    """The kernel forms of the large-level convolutions (tcgen05 with
    tensor-memory accumulators on every layer it takes, mma.sync on
    shared-memory tiles everywhere, and the default mix) give the same
    prediction on a grid of several tiles in every direction."""
    from ttcode_gb300 import guess
    from ttcode_gb300.fld import FLD
    from ttcode_gb300.grid import gitter
    from ttcode_gb300.synthetic import default_params
    X, Y, Z = 40, 64, 32
    f = FLD(gitter(X, Y, Z, 7.0e9, 7.7e9), default_params())
    guess.init(f, seed=5)
    rng = np.random.default_rng(1)
    feat = rng.uniform(-1, 1, (X * Y * Z, 5)).astype(np.float32)
    preds = []
    try:
        assert f.L.ttfld_guess_set_conv(3) == -1          # TTFLD_E_ARGS
        for form in (1, 0, 2):
            assert f.L.ttfld_guess_set_conv(form) == 0
            p = np.zeros(X * Y * Z, dtype=np.float32)
            assert f.L.ttfld_guess_predict(f.h, feat.ctypes.data, p.ctypes.data) == 0
            preds.append(p)
    finally:
        f.L.ttfld_guess_set_conv(2)   # the default form
    for p in (preds[0], preds[2]):
        assert np.linalg.norm(p - preds[1]) <= 1e-3 * np.linalg.norm(preds[1])


def test_seeded_training_is_reproducible():
    """The backward pass adds its partial sums in a fixed order (no floating-
    point atomics), so two trainings from the same seed on the same pairs give
    the same weights bit for bit, and the learned guess the same sweep count."""
    from ttcode_gb300 import guess
    from ttcode_gb300.fld import start_run
    from ttcode_gb300.synthetic import make_shell
    sh = make_shell(40, 64, 32, seed=2, delt=100.0)
    blobs, sweeps = [], []
    for _ in range(2):
        f = start_run(sh)
        guess.init(f, seed=1, capacity=4)
        assert guess.capture_pairs(f, sh, guess.random_cases(4, seed=10)) == 4
        for e in range(3):
            guess.train(f, epochs=1, lr=5e-4, seed=e)
        blobs.append(guess.save_weights(f))
        case = guess.random_cases(1, seed=99)[0]
        sweeps.append(guess.sweeps_with(f, sh, case, "learned")[0])
        f.close()
    assert blobs[0] == blobs[1]
    assert sweeps[0] == sweeps[1]
