"""Parity of the GPU push (cpic_push through the C ABI) against the oracle.

Exact variant (CPIC_PUSH_EXACT): particle state (offsets, momenta, cell
index) must be bit-identical, because the kernel and the oracle perform the
reference's arithmetic in the same order with separately rounded operations.
Default variant (fused multiply-adds, hardware reciprocal square root): every
particle within 1e-5 relative (the FP32 tolerance stated for this path), cell
indices equal except where a particle ends on a face.  Accumulators are sums
of the same terms in a different order (warp reductions and atomics), so they
must agree within the recursive-summation bound 2 (k-1) eps sum|x| per
accumulator (plus 1e-5 sum|x| for the default variant's per-term rounding).
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from support import assert_particles_close, random_state, reorder_bound  # noqa: E402

pytestmark = pytest.mark.gpu


def _run_pair(orc, st, true_sqrt=False, exact=True, tiles=True):
    from cabanapic_gb300 import pic
    R = st["real"]
    nc = st["num_cells"]
    host = st["particles"].copy()
    acc = np.zeros((nc, 3, 4), R)
    acc_abs = np.zeros((nc, 3, 4), R)
    cnt = np.zeros((nc, 3, 4), np.int32)
    crossers = orc.push(host, st["n"], st["vl"], st["interp"], *st["push_args"], acc, st["ogrid"],
                        acc_abs=acc_abs, acc_count=cnt, literal=not true_sqrt)
    P = pic.ParticleList(st["n"], R, st["vl"]).upload(st["particles"])
    I = pic.InterpolatorArray(nc, R)
    I.buf.copy_(torch.from_numpy(st["interp"]))
    A = pic.AccumulatorArray(nc, R)
    pic.push(P, I, *st["push_args"], A, None, st["nx"], st["ny"], st["nz"], 1, pic.Boundary.Periodic,
             true_sqrt=true_sqrt, exact=exact, tiles=tiles)
    pic.check_status()
    return host, acc, acc_abs, cnt, P.download_bytes(), A.get(), crossers


def _assert_parity(res, real, st=None, exact=True):
    host, acc, acc_abs, cnt, gpu_p, gpu_acc, _ = res
    eps = np.finfo(real).eps
    bound = reorder_bound(acc_abs, cnt, eps)
    if exact:
        assert np.array_equal(gpu_p, host), "particle AoSoA bytes differ from the oracle"
    else:
        assert_particles_close(gpu_p, host, st["n"], real, st["vl"], st["nx"], st["ny"], st["nz"])
        bound = bound + 1e-5 * acc_abs + 1e-6 * float(acc_abs.max())
    err = np.abs(gpu_acc.astype(np.float64) - acc.astype(np.float64))
    assert np.all(err <= bound), f"accumulator error {err.max():.3e} above the bound"


def _both(orc, st, real, **kw):
    _assert_parity(_run_pair(orc, st, exact=True, **kw), real, st, exact=True)
    _assert_parity(_run_pair(orc, st, exact=False, **kw), real, st, exact=False)


@pytest.mark.parametrize("sort", [False, True])
@pytest.mark.parametrize("n", [1, 31, 4000, 20011])
def test_push_float_vl32(orc, sort, n):
    st = random_state(nx=6, ny=5, nz=4, n=n, seed=n + int(sort), sort=sort)
    res = _run_pair(orc, st)
    _assert_parity(res, np.float32)
    _assert_parity(_run_pair(orc, st, exact=False), np.float32, st, exact=False)
    if n >= 4000:
        assert res[-1] > 0.2 * n  # the crossing path was exercised


@pytest.mark.parametrize("real,vl", [(np.float32, 32), (np.float32, 16), (np.float64, 32)])
@pytest.mark.parametrize("disorder", [0.0, 0.6])
def test_push_cell_window(orc, real, vl, disorder):
    """Particles in cell order on 40-cell rows at 64 per cell: a tile's run of
    cells fits the tiled kernel's shared-memory window, so window gathers serve
    nearly every particle.  With disorder, 60% of them sit in a neighbouring
    cell (as some steps after a sort): they still hit the window (one voxel of
    margin, y and z neighbour segments) except at its edges, where the global
    gather takes over.  Both kernels must match the oracle, and each other bit
    for bit in particle state."""
    st = random_state(nx=40, ny=3, nz=3, n=64 * 360, seed=7, real=real, vl=vl, sort=True,
                      crossing=0.05, disorder=disorder)
    _both(orc, st, real)
    _both(orc, st, real, tiles=False)
    tiled = _run_pair(orc, st, exact=False)
    stream = _run_pair(orc, st, exact=False, tiles=False)
    assert np.array_equal(tiled[4], stream[4])


def test_push_float_vl16(orc):
    st = random_state(nx=5, ny=4, nz=6, n=9999, seed=3, vl=16)
    _both(orc, st, np.float32)


@pytest.mark.parametrize("true_sqrt", [False, True])
def test_push_double(orc, true_sqrt):
    st = random_state(nx=4, ny=6, nz=5, n=6007, seed=11, real=np.float64)
    _both(orc, st, np.float64, true_sqrt=true_sqrt)


def test_push_collapsed_axes(orc):
    # a 1-D grid (ny = nz = 1), like the reference's 2stream decks
    st = random_state(nx=32, ny=1, nz=1, n=5000, seed=5, cdt=(0.5, 0.2, 0.2))
    _both(orc, st, np.float32)


def test_push_dense_cells_sorted(orc):
    # 64+ particles per cell in cell order: the warp-reduction path dominates
    st = random_state(nx=4, ny=4, nz=4, n=64 * 64 + 17, seed=9, sort=True, crossing=0.05)
    _both(orc, st, np.float32)


def test_push_accumulates_into_existing_values(orc):
    # push adds to the accumulator (ScatterView semantics): a non-zero start is kept
    from cabanapic_gb300 import pic
    st = random_state(n=3000, seed=21)
    nc = st["num_cells"]
    start = np.random.default_rng(0).standard_normal((nc, 3, 4)).astype(np.float32)
    host = st["particles"].copy()
    acc = start.copy()
    orc.push(host, st["n"], 32, st["interp"], *st["push_args"], acc, st["ogrid"])
    P = pic.ParticleList(st["n"], np.float32, 32).upload(st["particles"])
    I = pic.InterpolatorArray(nc, np.float32)
    I.buf.copy_(torch.from_numpy(st["interp"]))
    A = pic.AccumulatorArray(nc, np.float32)
    A.set(start)
    pic.push(P, I, *st["push_args"], A, None, st["nx"], st["ny"], st["nz"], 1, pic.Boundary.Periodic,
             exact=True)
    pic.check_status()
    assert np.allclose(A.get(), acc, rtol=1e-5, atol=1e-5)


def test_fast_and_exact_agree_on_a_thermal_plasma(orc):
    """Both variants on the benchmark's kind of input (sorted thermal plasma)."""
    from cabanapic_gb300 import decks, layout as L, pic
    deck = decks.thermal(n=12, ppc=32, num_steps=1, seed=5)
    p = deck.derived()
    host = L.pack_particles(decks.thermal_particles(deck), np.float32, 32)
    nc = deck.num_cells
    rng = np.random.default_rng(1)
    interp = L.pack_cells((rng.standard_normal((nc, 18)) * 0.05).astype(np.float32), np.float32)
    out = {}
    for exact in (True, False):
        P = pic.ParticleList(deck.num_particles, np.float32, 32).upload(host)
        I = pic.InterpolatorArray(nc, np.float32)
        I.buf.copy_(torch.from_numpy(interp))
        A = pic.AccumulatorArray(nc, np.float32)
        pic.push(P, I, p["qdt_2mc"], p["cdt_dx"], p["cdt_dy"], p["cdt_dz"], p["qsp"], A, None,
                 12, 12, 12, 1, pic.Boundary.Periodic, exact=exact)
        pic.check_status()
        out[exact] = (P.download_bytes(), A.get())
    ref = host.copy()
    acc = np.zeros((nc, 3, 4), np.float32)
    orc.push(ref, deck.num_particles, 32, interp, p["qdt_2mc"], p["cdt_dx"], p["cdt_dy"],
             p["cdt_dz"], p["qsp"], acc, orc.grid(12, 12, 12))
    assert np.array_equal(out[True][0], ref)
    assert_particles_close(out[False][0], ref, deck.num_particles, np.float32, 32, 12, 12, 12)


@pytest.mark.parametrize("tiles", [True, False])
def test_fp64_accumulation_bounds_hot_cell_error(orc, tiles):
    """CPIC_PUSH_ACC_F64: 8192 FP32 particles deposit into one cell.  The truth
    is the exact sum (math.fsum) of each particle's 12 FP32 deposits, taken
    from the oracle one particle at a time (the exact variant computes the
    same per-particle values).  With FP64 accumulator rows the GPU's error is
    the warps' FP32 tree alone (5 levels of 32 lanes), independent of the
    number of particles: at most 4 eps32 sum|x| per element."""
    import math
    from cabanapic_gb300 import layout as L, pic
    st = random_state(nx=4, ny=4, nz=4, n=8192, seed=17, crossing=0.0, edge_cases=False)
    R = np.float32
    h = {k: v.copy() for k, v in st["host"].items()}
    h["cell"][:] = L.voxel(2, 3, 2, 4, 4)
    rng = np.random.default_rng(3)
    for k in ("x", "y", "z"):
        h[k] = rng.uniform(-0.8, 0.8, 8192).astype(R)
    for k in ("ux", "uy", "uz"):
        h[k] = (rng.standard_normal(8192) * 0.05).astype(R)
    nc = st["num_cells"]
    cell = int(h["cell"][0])
    per = np.zeros((8192, 12))
    for i in range(8192):
        one = {k: v[i:i + 1] for k, v in h.items()}
        acc1 = np.zeros((nc, 3, 4), R)
        assert orc.push(L.pack_particles(one, R, 32), 1, 32, st["interp"], *st["push_args"], acc1, st["ogrid"]) == 0
        per[i] = acc1[cell].reshape(12)
    truth = np.array([math.fsum(per[:, k]) for k in range(12)])
    absum = np.abs(per).sum(axis=0)
    P = pic.ParticleList(8192, R, 32).upload(h)
    I = pic.InterpolatorArray(nc, R)
    I.buf.copy_(torch.from_numpy(st["interp"]))
    A64 = pic.AccumulatorArray(nc, np.float64)
    pic.push(P, I, *st["push_args"], A64, None, 4, 4, 4, 1, pic.Boundary.Periodic, exact=True, tiles=tiles)
    pic.check_status()
    got = A64.get()[cell].reshape(12)
    eps = np.finfo(np.float32).eps
    assert np.all(np.abs(got - truth) <= 4 * eps * absum), (np.abs(got - truth) / (eps * absum)).max()
    # the FP32 accumulator sums the same warp totals in float; record its error for comparison
    P32 = pic.ParticleList(8192, R, 32).upload(h)
    A32 = pic.AccumulatorArray(nc, R)
    pic.push(P32, I, *st["push_args"], A32, None, 4, 4, 4, 1, pic.Boundary.Periodic, exact=True, tiles=tiles)
    pic.check_status()
    err32 = np.abs(A32.get()[cell].reshape(12).astype(np.float64) - truth) / (eps * absum)
    assert np.all(err32 <= 2 * 8192 / 32)  # the recursive-summation bound over the warp totals
    # the particle states are the same as with FP32 accumulators
    assert np.array_equal(P.download_bytes(), P32.download_bytes())


@pytest.mark.parametrize("real,vl,acc64", [(np.float32, 32, False), (np.float32, 16, False), (np.float64, 32, False),
                                            (np.float32, 32, True)])
def test_push_into_matches_in_place_push(orc, real, vl, acc64):
    """cpic_push_into: the out-of-place push writes exactly the in-place push's
    particle bytes (all members, skipped particles copied unchanged) into the
    second list and leaves the source untouched; the deposits agree within
    the summation-order bound."""
    from cabanapic_gb300 import layout as L, pic
    st = random_state(nx=7, ny=6, nz=5, n=30011, seed=31, real=real, vl=vl, crossing=0.2, sort=True,
                      disorder=0.2)
    host = dict(st["host"])
    host["cell"] = host["cell"].copy()
    host["cell"][[3, 777]] = [-2, st["num_cells"] + 4]  # skipped and reported
    packed = L.pack_particles(host, real, vl)
    nc = st["num_cells"]
    # the oracle (like the reference) has no range check: it pushes the two
    # with valid cells and zero weight (no deposit), and the expected list
    # then holds them unchanged
    ok = {k: v.copy() for k, v in host.items()}
    ok["cell"][[3, 777]] = st["host"]["cell"][[3, 777]]
    ok["w"][[3, 777]] = 0
    ref_p = L.pack_particles(ok, real, vl)
    acc = np.zeros((nc, 3, 4), real)
    acc_abs = np.zeros_like(acc)
    cnt = np.zeros((nc, 3, 4), np.int32)
    orc.push(ref_p, st["n"], vl, st["interp"], *st["push_args"], acc, st["ogrid"], acc_abs=acc_abs, acc_count=cnt)
    out = L.unpack_particles(ref_p, st["n"], real, vl)
    for k in out:
        out[k][[3, 777]] = host[k][[3, 777]]
    ref = L.pack_particles(out, real, vl)
    P = pic.ParticleList(st["n"], real, vl).upload(packed)
    Q = pic.ParticleList(st["n"], real, vl)
    Q.buf.fill_(0xAB)
    I = pic.InterpolatorArray(nc, real)
    I.buf.copy_(torch.from_numpy(st["interp"]))
    A = pic.AccumulatorArray(nc, np.float64 if acc64 else real)  # FP64 rows: CPIC_PUSH_ACC_F64
    pic.push_into(P, Q, I, *st["push_args"], A, None, 7, 6, 5, 1, pic.Boundary.Periodic, exact=True)
    with pytest.raises(Exception):
        pic.check_status()  # the two out-of-range cells are reported
    assert np.array_equal(P.download_bytes(), packed)
    # every member of every particle (the padding slots of the last block are not written)
    got, want = L.unpack_particles(Q.download_bytes(), st["n"], real, vl), L.unpack_particles(ref, st["n"], real, vl)
    for k in want:
        assert np.array_equal(got[k].view(np.uint8), want[k].view(np.uint8)), k
    eps = np.finfo(real).eps
    assert np.all(np.abs(A.get().astype(np.float64) - acc) <= reorder_bound(acc_abs, cnt, eps))


@pytest.mark.parametrize("tiles", [True, False])
@pytest.mark.parametrize("real", [np.float32, np.float64])
def test_push_accumulator_layout_left(orc, tiles, real):
    """CPIC_PUSH_ACC_LAYOUT_LEFT: the accumulator in Kokkos' LayoutLeft, the
    default layout of accumulator_array_t = View<real_t*[3][4]> in a Kokkos-Cuda
    build of the reference (src/types.h:120, example/example.cpp:137).  The
    particles are the LayoutRight push's bytes; the deposits, read back
    transposed, are the oracle's within the summation-reordering bound."""
    from cabanapic_gb300 import pic
    st = random_state(nx=7, ny=5, nz=4, n=20011, seed=23, real=real, sort=True, crossing=0.2, disorder=0.3)
    nc = st["num_cells"]
    host = st["particles"].copy()
    acc = np.zeros((nc, 3, 4), real)
    acc_abs = np.zeros_like(acc)
    cnt = np.zeros((nc, 3, 4), np.int32)
    orc.push(host, st["n"], st["vl"], st["interp"], *st["push_args"], acc, st["ogrid"], acc_abs=acc_abs,
             acc_count=cnt)
    for exact in (True, False):
        P = pic.ParticleList(st["n"], real, st["vl"]).upload(st["particles"])
        I = pic.InterpolatorArray(nc, real)
        I.buf.copy_(torch.from_numpy(st["interp"]))
        A = pic.AccumulatorArray(nc, real, layout="left")
        pic.push(P, I, *st["push_args"], A, None, st["nx"], st["ny"], st["nz"], 1, pic.Boundary.Periodic,
                 exact=exact, tiles=tiles)
        pic.check_status()
        bound = reorder_bound(acc_abs, cnt, np.finfo(real).eps)
        if exact:
            assert np.array_equal(P.download_bytes(), host)
        else:
            assert_particles_close(P.download_bytes(), host, st["n"], real, st["vl"], st["nx"], st["ny"], st["nz"])
            bound = bound + 1e-5 * acc_abs + 1e-6 * float(acc_abs.max())
        err = np.abs(A.get().astype(np.float64) - acc)
        assert np.all(err <= bound), err.max()
