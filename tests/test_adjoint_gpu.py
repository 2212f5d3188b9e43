"""The adjoint step: transposed field kernels (dot-product identities against
the forward kernels), the push adjoint against FP64 central differences of
the oracle's push, and whole-run gradients of the field energy against FP64
finite differences of the forward run."""
import ctypes as C

import numpy as np
import pytest

torch = pytest.importorskip("torch")

from support import random_state  # noqa: E402

pytestmark = pytest.mark.gpu

GRIDS = [(6, 5, 4), (1, 16, 1), (7, 1, 3)]


def _periodic_fill(cells, nx, ny, nz):
    """cells (num_cells, 9): set every ghost cell to its periodic image."""
    a = cells.reshape(nz + 2, ny + 2, nx + 2, -1)
    a[:, :, 0] = a[:, :, nx]; a[:, :, nx + 1] = a[:, :, 1]
    a[:, 0, :] = a[:, ny, :]; a[:, ny + 1, :] = a[:, 1, :]
    a[0, :, :] = a[nz, :, :]; a[nz + 1, :, :] = a[1, :, :]
    return cells


def _interior(cells, nx, ny, nz):
    return cells.reshape(nz + 2, ny + 2, nx + 2, -1)[1:-1, 1:-1, 1:-1]


def _lib():
    from cabanapic_gb300 import capi
    return capi.load()


def _fa(vals, nc, real=np.float64):
    from cabanapic_gb300 import pic
    F = pic.FieldArray(nc, real)
    F.set_members(vals)
    return F


@pytest.mark.parametrize("g", GRIDS)
def test_adjoint_advance_b_is_the_transpose(g):
    from cabanapic_gb300 import capi, pic
    nx, ny, nz = g
    nc = (nx + 2) * (ny + 2) * (nz + 2)
    rng = np.random.default_rng(1)
    v = _periodic_fill(rng.standard_normal((nc, 9)), nx, ny, nz)
    lam = rng.standard_normal((nc, 9))
    lam[:, 0:3] = 0
    pxyz = [0.3 if n > 1 else 0.0 for n in g]
    F = _fa(v, nc)
    pic.EMFieldSolver().advance_b(F, *pxyz, nx, ny, nz, 1)
    dB = _interior(F.get_members() - v, nx, ny, nz)[..., 3:6]
    LF = _fa(lam, nc)
    _lib().call("cpic_adjoint_advance_b", LF.ptr, *pxyz, C.byref(capi.make_grid(nx, ny, nz)), 8, None)
    lE = _interior(LF.get_members(), nx, ny, nz)[..., 0:3]
    lhs = np.sum(_interior(lam, nx, ny, nz)[..., 3:6] * dB)
    rhs = np.sum(lE * _interior(v, nx, ny, nz)[..., 0:3])
    assert np.isclose(lhs, rhs, rtol=1e-12, atol=1e-12)


@pytest.mark.parametrize("g", GRIDS)
def test_adjoint_advance_e_is_the_transpose(g):
    from cabanapic_gb300 import capi, pic
    nx, ny, nz = g
    nc = (nx + 2) * (ny + 2) * (nz + 2)
    rng = np.random.default_rng(2)
    v = _periodic_fill(rng.standard_normal((nc, 9)), nx, ny, nz)
    J = np.zeros((nc, 3))
    _interior(J, nx, ny, nz)[...] = rng.standard_normal((nz, ny, nx, 3))
    v[:, 6:9] = J  # jf on the interior only: the fold adds nothing, the copy fills ghosts
    lam = np.zeros((nc, 9))
    lam[:, 0:3] = rng.standard_normal((nc, 3))
    pxyz = [0.3 if n > 1 else 0.0 for n in g]
    cj = 0.07
    F = _fa(v, nc)
    pic.EMFieldSolver().advance_e(F, *pxyz, nx, ny, nz, 1, cj)
    dE = _interior(F.get_members() - v, nx, ny, nz)[..., 0:3]
    LF = _fa(lam, nc)
    _lib().call("cpic_adjoint_advance_e", LF.ptr, *pxyz, C.byref(capi.make_grid(nx, ny, nz)), cj, 8, None)
    out = _interior(LF.get_members(), nx, ny, nz)
    lhs = np.sum(_interior(lam, nx, ny, nz)[..., 0:3] * dE)
    rhs = np.sum(out[..., 3:6] * _interior(v, nx, ny, nz)[..., 3:6]) + np.sum(out[..., 6:9] * _interior(J, nx, ny, nz))
    assert np.isclose(lhs, rhs, rtol=1e-12, atol=1e-12)


@pytest.mark.parametrize("g", GRIDS)
def test_adjoint_unload_is_the_transpose(orc, g):
    from cabanapic_gb300 import capi, layout as L, pic
    nx, ny, nz = g
    nc = (nx + 2) * (ny + 2) * (nz + 2)
    rng = np.random.default_rng(3)
    acc = np.zeros((nc, 3, 4))
    _interior(acc.reshape(nc, 12), nx, ny, nz)[...] = rng.standard_normal((nz, ny, nx, 12))
    dx, dy, dz, dt = 0.3, 0.25, 0.2, 0.07
    # forward: unload, then the periodic fold of advance_e (oracle's current_fold)
    F = pic.FieldArray(nc, np.float64)
    A = pic.AccumulatorArray(nc, np.float64)
    A.set(acc)
    pic.unload_accumulator_array(F, A, nx, ny, nz, 1, dx, dy, dz, dt)
    f = F.buf.cpu().numpy().copy()
    orc.current_fold(f, orc.grid(nx, ny, nz))
    J = _interior(L.unpack_cells(f, nc, 9), nx, ny, nz)[..., 6:9]
    lamJ = np.zeros((nc, 9))
    _interior(lamJ, nx, ny, nz)[..., 6:9] = rng.standard_normal((nz, ny, nx, 3))
    LF = _fa(lamJ, nc)
    LA = pic.AccumulatorArray(nc, np.float64)
    _lib().call("cpic_adjoint_unload_accumulator", LF.ptr, LA.ptr, C.byref(capi.make_grid(nx, ny, nz)),
                dx, dy, dz, dt, 8, None)
    la = _interior(LA.get().reshape(nc, 12), nx, ny, nz)
    lhs = np.sum(_interior(lamJ, nx, ny, nz)[..., 6:9] * J)
    rhs = np.sum(la * _interior(acc.reshape(nc, 12), nx, ny, nz))
    assert np.isclose(lhs, rhs, rtol=1e-12, atol=1e-12)


@pytest.mark.parametrize("g", GRIDS)
def test_adjoint_interpolator_is_the_transpose(g):
    from cabanapic_gb300 import capi, layout as L, pic
    nx, ny, nz = g
    nc = (nx + 2) * (ny + 2) * (nz + 2)
    rng = np.random.default_rng(4)
    v = _periodic_fill(rng.standard_normal((nc, 9)), nx, ny, nz)
    F = _fa(v, nc)
    I = pic.InterpolatorArray(nc, np.float64)
    pic.load_interpolator_array(F, I, nx, ny, nz, 1)
    Iv = _interior(I.get_members(), nx, ny, nz)
    lamI = np.zeros((nc, 18))
    _interior(lamI, nx, ny, nz)[...] = rng.standard_normal((nz, ny, nx, 18))
    LI = pic.InterpolatorArray(nc, np.float64)
    LI.set_members(lamI)
    LF = pic.FieldArray(nc, np.float64)
    _lib().call("cpic_adjoint_load_interpolator", LI.ptr, LF.ptr, C.byref(capi.make_grid(nx, ny, nz)), 8, None)
    lhs = np.sum(_interior(lamI, nx, ny, nz) * Iv)
    rhs = np.sum(_interior(LF.get_members(), nx, ny, nz)[..., 0:6] * _interior(v, nx, ny, nz)[..., 0:6])
    assert np.isclose(lhs, rhs, rtol=1e-12, atol=1e-12)


def _push_objective(orc, st, packed, lam_p, lam_a):
    """g = <lambda_P', P'> + <lambda_a, a> for the oracle's FP64 push (sqrt for gamma)."""
    from cabanapic_gb300 import layout as L
    buf = packed.copy()
    acc = np.zeros((st["num_cells"], 3, 4))
    orc.push(buf, st["n"], 32, st["interp"], *st["push_args"], acc, st["ogrid"], literal=False)
    out = L.unpack_particles(buf, st["n"], np.float64, 32)
    g = sum(np.sum(lam_p[k] * out[k]) for k in ("x", "y", "z", "ux", "uy", "uz"))
    return g + np.sum(lam_a * acc), out["cell"]


@pytest.mark.parametrize("crossing", [0.0, 0.5])
def test_adjoint_push_matches_central_differences(orc, crossing):
    from cabanapic_gb300 import capi, layout as L, pic
    st = random_state(nx=5, ny=4, nz=4, n=64, seed=21, real=np.float64, crossing=crossing, edge_cases=False)
    nc, n = st["num_cells"], st["n"]
    rng = np.random.default_rng(5)
    keys = ("x", "y", "z", "ux", "uy", "uz")
    lam_p = {k: rng.standard_normal(n) for k in keys}
    lam_a = rng.standard_normal((nc, 3, 4))
    # adjoint on the GPU
    P = pic.ParticleList(n, np.float64, 32).upload(st["particles"])
    I = pic.InterpolatorArray(nc, np.float64)
    I.buf.copy_(torch.from_numpy(st["interp"]))
    LA = pic.AccumulatorArray(nc, np.float64)
    LA.set(lam_a)
    lp = dict(lam_p, w=np.zeros(n), cell=np.zeros(n, np.int32))
    LP = pic.ParticleList(n, np.float64, 32).upload(lp)
    LI = pic.InterpolatorArray(nc, np.float64)
    prm = capi.CpicPushParams(*[float(v) for v in st["push_args"]], 8, 32, capi.CPIC_PUSH_TRUE_SQRT, 0)
    _lib().call("cpic_adjoint_push", P.ptr, n, I.ptr, LA.ptr, LP.ptr, LI.ptr,
                C.byref(capi.make_grid(st["nx"], st["ny"], st["nz"])), C.byref(prm),
                pic.status_word().data_ptr(), None)
    pic.check_status()
    grad = LP.download()
    # central differences of the oracle's push, one particle component at a time
    h = 1e-6
    base = st["host"]
    checked = 0
    for pidx in range(0, n, 5):
        for k in keys:
            hp = {kk: vv.copy() for kk, vv in base.items()}
            hm = {kk: vv.copy() for kk, vv in base.items()}
            hp[k][pidx] += h
            hm[k][pidx] -= h
            gp, cp = _push_objective(orc, st, L.pack_particles(hp, np.float64, 32), lam_p, lam_a)
            gm, cm = _push_objective(orc, st, L.pack_particles(hm, np.float64, 32), lam_p, lam_a)
            if not np.array_equal(cp, cm):
                continue  # the perturbation changed a cell index: not differentiable here
            fd = (gp - gm) / (2 * h)
            assert abs(grad[k][pidx] - fd) <= 1e-6 * max(1.0, abs(fd)), (pidx, k, grad[k][pidx], fd)
            checked += 1
    assert checked > 50
    # the interpolator adjoint: perturb coefficients of one populated cell
    cell = int(base["cell"][0])
    lam_I = LI.get_members()
    for m in (0, 3, 6, 9, 12, 13, 17):
        ip = st["interp"].copy()
        im = st["interp"].copy()
        off = (cell // 32) * 18 * 32 + m * 32 + cell % 32
        ip[off] += h
        im[off] -= h
        gp, _ = _push_objective(orc, dict(st, interp=ip), st["particles"], lam_p, lam_a)
        gm, _ = _push_objective(orc, dict(st, interp=im), st["particles"], lam_p, lam_a)
        fd = (gp - gm) / (2 * h)
        assert abs(lam_I[cell, m] - fd) <= 1e-6 * max(1.0, abs(fd)), (m, lam_I[cell, m], fd)


def _two_stream_loss(deck, host, K, precision=8):
    from cabanapic_gb300.adjoint import AdjointRun
    run = AdjointRun(deck, host, checkpoint=10, true_sqrt=True, exact=True)
    return run.forward(K)


@pytest.mark.parametrize("precision,tol", [(8, 1e-6), (4, 1e-3)])
def test_two_stream_gradients_match_fp64_finite_differences(precision, tol):
    """dL/d(drift), dL/d(perturbation amplitude) and dL/du for a few initial
    momenta, L = field energy after K = 30 steps of a 32-cell two-stream run;
    FP64 central differences of the FP64 GPU forward.

    The loss is only piecewise smooth: the interpolated E_x is constant in x
    inside a cell (src/push.h:124-126), so it jumps when a particle
    crosses a face.  A step h large enough that the +h and -h runs differ in
    the step at which some particle crosses a face measures the jump, not the
    derivative: at K = 30, h = 1e-6 and 1e-5 do (the central difference even
    changes sign), while h = 1e-7 and 1e-8 agree with each other and with the
    adjoint to ~1e-9.  So h = 1e-7, and the test also checks that h and h/4
    agree, which fails if a crossing falls between them."""
    from cabanapic_gb300 import decks
    from cabanapic_gb300.adjoint import AdjointRun, two_stream_drift_gradients
    K = 30

    def setup(prec, drift=0.2, amp=1e-3):
        d = decks.two_stream_1d(precision=prec, nx=32, ppc_per_beam=32, num_steps=K, drift=drift, amp=amp)
        return d, decks.two_stream_1d_particles(d)

    deck, host = setup(precision)
    run = AdjointRun(deck, host, checkpoint=10, true_sqrt=(precision == 8), exact=True)
    run.forward(K)
    lam, _ = run.backward()
    g_drift, g_amp = two_stream_drift_gradients(lam, deck, host)
    h = 1e-7

    def fd_param(name, v0, hh):
        return (_two_stream_loss(*setup(8, **{name: v0 + hh}), K)
                - _two_stream_loss(*setup(8, **{name: v0 - hh}), K)) / (2 * hh)

    fd_drift, fd_amp = fd_param("drift", 0.2, h), fd_param("amp", 1e-3, h)
    assert abs(fd_param("drift", 0.2, h / 4) - fd_drift) <= 1e-6 * abs(fd_drift)
    assert abs(g_drift - fd_drift) <= tol * abs(fd_drift), (g_drift, fd_drift)
    assert abs(g_amp - fd_amp) <= tol * abs(fd_amp) + 1e-3 * tol * abs(fd_drift), (g_amp, fd_amp)
    # a few individual initial momenta
    d64, h64 = setup(8)
    for pidx in (0, 17, 1000, 2047):
        hp = {k: v.copy() for k, v in h64.items()}
        hm = {k: v.copy() for k, v in h64.items()}
        hp["ux"][pidx] += h
        hm["ux"][pidx] -= h
        fd = (_two_stream_loss(d64, hp, K) - _two_stream_loss(d64, hm, K)) / (2 * h)
        assert abs(lam["ux"][pidx] - fd) <= tol * max(abs(fd), 1e-3 * abs(fd_drift) / 2048), (pidx, lam["ux"][pidx], fd)


def test_uniform_ex_gradient_3d_matches_fp64_finite_differences():
    """dL/dE0 for a uniform initial E_x = E0 in an 8^3 x 8 ppc thermal plasma, K = 20."""
    from cabanapic_gb300 import decks
    from cabanapic_gb300.adjoint import AdjointRun
    K = 20

    def fields(deck, E0):
        f = np.zeros((deck.num_cells, 9))
        f[:, 0] = E0
        return f

    def loss(E0):
        d = decks.thermal(n=8, ppc=8, uth=0.1, dx=0.1, precision=8, num_steps=K, seed=3)
        r = AdjointRun(d, decks.thermal_particles(d), fields_init=fields(d, E0), checkpoint=7,
                       true_sqrt=True, exact=True)
        return r.forward(K)

    d = decks.thermal(n=8, ppc=8, uth=0.1, dx=0.1, precision=8, num_steps=K, seed=3)
    run = AdjointRun(d, decks.thermal_particles(d), fields_init=fields(d, 0.01), checkpoint=7,
                     true_sqrt=True, exact=True)
    run.forward(K)
    _, lamF = run.backward()
    g = float(_interior(lamF, 8, 8, 8)[..., 0].sum())
    h = 1e-6
    fd = (loss(0.01 + h) - loss(0.01 - h)) / (2 * h)
    assert abs(g - fd) <= 1e-6 * abs(fd), (g, fd)


def test_adjoint_interpolator_scatter_independent_of_particle_order():
    """The transpose of the gather is reduced over the warp's largest group of
    lanes sharing a cell: with particles in cell order (whole warps in one
    cell) and the same particles shuffled (groups of one or two), the
    per-particle adjoints are identical and the interpolator adjoint agrees
    to FP64 summation-order precision."""
    from cabanapic_gb300 import capi, layout as L, pic
    st = random_state(nx=6, ny=5, nz=4, n=6000, seed=8, real=np.float64, crossing=0.1, sort=True)
    nc, n = st["num_cells"], st["n"]
    rng = np.random.default_rng(2)
    lam_a = rng.standard_normal((nc, 3, 4))
    lam_p = {k: rng.standard_normal(n) for k in ("x", "y", "z", "ux", "uy", "uz")}
    perm = rng.permutation(n)

    def run(order):
        host = {k: v[order] for k, v in st["host"].items()}
        P = pic.ParticleList(n, np.float64, 32).upload(host)
        I = pic.InterpolatorArray(nc, np.float64)
        I.buf.copy_(torch.from_numpy(st["interp"]))
        LA = pic.AccumulatorArray(nc, np.float64)
        LA.set(lam_a)
        LP = pic.ParticleList(n, np.float64, 32).upload(
            dict({k: v[order] for k, v in lam_p.items()}, w=np.zeros(n), cell=np.zeros(n, np.int32)))
        LI = pic.InterpolatorArray(nc, np.float64)
        prm = capi.CpicPushParams(*[float(v) for v in st["push_args"]], 8, 32, capi.CPIC_PUSH_TRUE_SQRT, 0)
        _lib().call("cpic_adjoint_push", P.ptr, n, I.ptr, LA.ptr, LP.ptr, LI.ptr,
                    C.byref(capi.make_grid(st["nx"], st["ny"], st["nz"])), C.byref(prm),
                    pic.status_word().data_ptr(), None)
        pic.check_status()
        return LP.download(), LI.get_members()

    lp_a, li_a = run(np.arange(n))
    lp_b, li_b = run(perm)
    inv = np.argsort(perm)
    for k in ("x", "y", "z", "ux", "uy", "uz"):
        assert np.array_equal(lp_a[k], lp_b[k][inv]), k
    scale = np.abs(li_a).max()
    np.testing.assert_allclose(li_b, li_a, rtol=0, atol=1e-12 * scale)
    assert scale > 0


@pytest.mark.parametrize("case", ["two-stream", "thermal3d"])
def test_fp32_adjoint_matches_fp64_gpu_adjoint(case):
    """The FP32 adjoint against the FP64 GPU adjoint of the same initial state
    (the FP32 particles cast to FP64): the parameter gradients within 1e-3,
    and the per-particle momentum adjoints within 1e-3 of their scale (all
    but a few particles per thousand)."""
    from cabanapic_gb300 import decks
    from cabanapic_gb300.adjoint import AdjointRun, two_stream_drift_gradients
    out = {}
    for prec in (4, 8):
        if case == "two-stream":
            K = 40
            d = decks.two_stream_1d(precision=prec, nx=32, ppc_per_beam=32, num_steps=K)
            host = decks.two_stream_1d_particles(decks.two_stream_1d(precision=4, nx=32, ppc_per_beam=32))
            host = {k: (v.astype(d.R) if k not in ("cell", "X", "sign") else v) for k, v in host.items()}
            run = AdjointRun(d, host, checkpoint=10)
            run.forward(K)
            lam, _ = run.backward()
            out[prec] = (np.array(two_stream_drift_gradients(lam, d, host)), lam["ux"].astype(np.float64))
        else:
            K = 12
            d = decks.thermal(n=12, ppc=8, uth=0.1, dx=0.1, precision=prec, num_steps=K, seed=4)
            host = decks.thermal_particles(decks.thermal(n=12, ppc=8, uth=0.1, dx=0.1, precision=4, seed=4))
            host = {k: (v.astype(d.R) if k != "cell" else v) for k, v in host.items()}
            f = np.zeros((d.num_cells, 9))
            f[:, 0] = 0.02
            run = AdjointRun(d, host, fields_init=f, checkpoint=5)
            run.forward(K)
            lam, lamF = run.backward()
            a = lamF.reshape(d.nz + 2, d.ny + 2, d.nx + 2, 9)[1:-1, 1:-1, 1:-1]
            out[prec] = (np.array([a[..., 0].sum()]), lam["ux"].astype(np.float64))
    (g32, u32), (g64, u64) = out[4], out[8]
    np.testing.assert_allclose(g32, g64, rtol=1e-3)
    # a particle whose FP32 and FP64 runs cross a face at different steps has
    # a different (piecewise constant) path: allow a few in a thousand
    close = np.abs(u32 - u64) <= 1e-3 * np.abs(u64).max()
    assert close.mean() >= 0.995, close.mean()


@pytest.mark.parametrize("precision,tol", [(8, 1e-5), (4, 1e-3)])
def test_two_stream_256_cells_gradients_at_full_size(orc, precision, tol):
    """The adjoint configuration's two-stream case at its own size: 256 cells,
    256 particles per cell per beam (131,072 particles), checkpoints every 20
    steps; the gradients of the field energy after K = 50 steps with respect
    to the beam drift, the perturbation amplitude and a few initial momenta,
    against FP64 central differences of the oracle (the reference's step in
    FP64 with sqrt for gamma, deterministic): FP64 adjoint within 1e-5, FP32
    adjoint within 1e-3.  The differences use steps of 1e-9 and below, where
    two consecutive sizes agree (larger steps straddle the loss's jumps)."""
    from cabanapic_gb300 import decks, layout as L
    from cabanapic_gb300.adjoint import AdjointRun, two_stream_drift_gradients
    from support import oracle_loss, robust_central_difference
    K = 50

    def setup(prec, drift=0.2, amp=1e-3):
        d = decks.two_stream_1d(precision=prec, nx=256, ppc_per_beam=256, num_steps=K, drift=drift, amp=amp)
        return d, decks.two_stream_1d_particles(d)

    def loss(**kw):
        d, h = setup(8, **kw)
        return oracle_loss(orc, d, L.pack_particles(h, np.float64, 32), K, literal=False)

    deck, host = setup(precision)
    assert deck.num_particles == 131072
    run = AdjointRun(deck, host, checkpoint=20, true_sqrt=(precision == 8), exact=True)
    run.forward(K)
    lam, _ = run.backward()
    g_drift, g_amp = two_stream_drift_gradients(lam, deck, host)
    hs = [1e-9, 5e-10, 2.5e-10, 1e-10]
    fd_drift, _ = robust_central_difference(lambda v: loss(drift=v), 0.2, hs)
    fd_amp, _ = robust_central_difference(lambda v: loss(amp=v), 1e-3, hs, agree=1e-4)
    assert abs(g_drift - fd_drift) <= tol * abs(fd_drift), (g_drift, fd_drift)
    assert abs(g_amp - fd_amp) <= tol * abs(fd_amp) + 1e-3 * tol * abs(fd_drift), (g_amp, fd_amp)
    # individual initial momenta
    d64, h64 = setup(8)
    for pidx in (5, 70001, 131071):
        def loss_u(v, pidx=pidx):
            hp = {k: a.copy() for k, a in h64.items()}
            hp["ux"][pidx] = v
            return oracle_loss(orc, d64, L.pack_particles(hp, np.float64, 32), K, literal=False)
        fd, _ = robust_central_difference(loss_u, float(h64["ux"][pidx]), [1e-8, 5e-9, 2.5e-9], agree=1e-4)
        assert abs(lam["ux"][pidx] - fd) <= tol * max(abs(fd), 1e-3 * abs(fd_drift) / deck.num_particles), \
            (pidx, lam["ux"][pidx], fd)


@pytest.mark.parametrize("precision,tol", [(8, 2e-5), (4, 1e-3)])
def test_uniform_ex_gradient_64_cubed_at_full_size(orc, precision, tol):
    """The adjoint configuration's 3-D case at its own size: a 64^3 x 16 ppc
    thermal plasma (4,194,304 particles), uniform initial E_x = E0 = 0.01,
    K = 50, checkpoints every 20 steps: dL/dE0 against FP64 central
    differences of the oracle (sqrt for gamma, deterministic; steps of 1e-10
    and below agree, 1e-9 straddles a jump): FP64 adjoint within 2e-5, FP32
    adjoint within 1e-3."""
    from cabanapic_gb300 import decks, layout as L
    from cabanapic_gb300.adjoint import AdjointRun
    from support import oracle_loss, robust_central_difference
    K = 50

    def deck(prec):
        return decks.thermal(n=64, ppc=16, precision=prec, num_steps=K)

    def fields(d, E0):
        f = np.zeros((d.num_cells, 9))
        f[:, 0] = E0
        return f

    d64 = deck(8)
    packed64 = orc.thermal_particles(d64)
    fd, _ = robust_central_difference(
        lambda e0: oracle_loss(orc, d64, packed64, K, fields_init=fields(d64, e0), literal=False),
        0.01, [1e-10, 5e-11, 2.5e-11])
    d = deck(precision)
    host = L.unpack_particles(orc.thermal_particles(d), d.num_particles, d.R, d.vl)
    run = AdjointRun(d, host, fields_init=fields(d, 0.01), checkpoint=20, true_sqrt=(precision == 8),
                     exact=True)
    run.forward(K)
    _, lamF = run.backward()
    g = float(_interior(lamF, 64, 64, 64)[..., 0].sum())
    assert abs(g - fd) <= tol * abs(fd), (g, fd)


@pytest.mark.parametrize("real", [np.float64, np.float32])
def test_adjoint_interpolator_rows_layout(real):
    """CPIC_ADJ_INTERP_ROWS: the push adjoint adds each cell's 18 coefficient
    adjoints into a cell-major row instead of the interpolator's AoSoA layout,
    and cpic_adjoint_load_interpolator_rows transposes the interpolator load
    from that layout.  The particle adjoints are identical; the field adjoint
    equals the AoSoA pair's to summation-order precision."""
    from cabanapic_gb300 import capi, pic
    st = random_state(nx=6, ny=5, nz=4, n=20000, seed=12, real=real, crossing=0.2, sort=True, disorder=0.3)
    nc, n = st["num_cells"], st["n"]
    rng = np.random.default_rng(6)
    lam_p = {k: rng.standard_normal(n).astype(real) for k in ("x", "y", "z", "ux", "uy", "uz")}
    lam_a = rng.standard_normal((nc, 3, 4)).astype(real)
    prec = np.dtype(real).itemsize
    grid = capi.make_grid(st["nx"], st["ny"], st["nz"])
    out = []
    for rows in (False, True):
        P = pic.ParticleList(n, real, 32).upload(st["particles"])
        I = pic.InterpolatorArray(nc, real)
        I.buf.copy_(torch.from_numpy(st["interp"]))
        LA = pic.AccumulatorArray(nc, real)
        LA.set(lam_a)
        LP = pic.ParticleList(n, real, 32).upload(dict(lam_p, w=np.zeros(n, real), cell=np.zeros(n, np.int32)))
        flags = (capi.CPIC_PUSH_TRUE_SQRT if prec == 8 else 0) | (capi.CPIC_ADJ_INTERP_ROWS if rows else 0)
        prm = capi.CpicPushParams(*[float(v) for v in st["push_args"]], prec, 32, flags, 0)
        if rows:
            LI = torch.zeros(nc * capi.CPIC_ADJ_INTERP_ROW, dtype=I.buf.dtype, device="cuda")
            li_ptr = LI.data_ptr()
        else:
            LI = pic.InterpolatorArray(nc, real)
            li_ptr = LI.ptr
        _lib().call("cpic_adjoint_push", P.ptr, n, I.ptr, LA.ptr, LP.ptr, li_ptr, C.byref(grid), C.byref(prm),
                    pic.status_word().data_ptr(), None)
        pic.check_status()
        LF = _fa(np.zeros((nc, 9)), nc, real)
        fn = "cpic_adjoint_load_interpolator_rows" if rows else "cpic_adjoint_load_interpolator"
        _lib().call(fn, li_ptr, LF.ptr, C.byref(grid), prec, None)
        out.append((LP.download_bytes(), _interior(LF.get_members(), st["nx"], st["ny"], st["nz"])))
    assert np.array_equal(out[0][0], out[1][0])
    a, b = out[0][1].astype(np.float64), out[1][1].astype(np.float64)
    tol = 1e-10 if real == np.float64 else 1e-4
    assert np.abs(a - b).max() <= tol * np.abs(a).max(), np.abs(a - b).max() / np.abs(a).max()
