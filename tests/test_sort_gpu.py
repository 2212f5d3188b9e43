"""The counting sort by cell: keys sorted, particle records preserved, and the
push after a sort still matches the oracle on the sorted array."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from support import random_state, reorder_bound  # noqa: E402

pytestmark = pytest.mark.gpu


def _records(p):
    keys = [p["cell"]] + [p[k].view(np.uint32 if p[k].dtype == np.float32 else np.uint64)
                          for k in ("x", "y", "z", "ux", "uy", "uz", "w")]
    return np.lexsort(keys[::-1]), keys


@pytest.mark.parametrize("real,vl", [(np.float32, 32), (np.float32, 16), (np.float64, 32)])
@pytest.mark.parametrize("n", [1, 100, 50021])
def test_sort_permutes_into_cell_order(real, vl, n):
    from cabanapic_gb300 import pic
    st = random_state(nx=9, ny=7, nz=5, n=n, seed=n, real=real, vl=vl)
    P = pic.ParticleList(n, real, vl).upload(st["particles"])
    pic.sort_particles(P, st["num_cells"])
    out = P.download()
    assert np.all(np.diff(out["cell"]) >= 0)
    # same multiset of particle records
    a = st["host"]
    ia, ka = _records(a)
    ib, kb = _records(out)
    for x, y in zip(ka, kb):
        assert np.array_equal(x[ia], y[ib])


def test_sort_then_push_matches_oracle(orc):
    from cabanapic_gb300 import pic
    st = random_state(nx=8, ny=8, nz=8, n=40000, seed=4, crossing=0.1)
    nc = st["num_cells"]
    P = pic.ParticleList(st["n"], np.float32, 32).upload(st["particles"])
    sorter = pic.Sorter(P, nc)
    sorter(P)
    sorted_bytes = P.download_bytes()
    host = sorted_bytes.copy()
    acc = np.zeros((nc, 3, 4), np.float32)
    acc_abs = np.zeros_like(acc)
    cnt = np.zeros((nc, 3, 4), np.int32)
    orc.push(host, st["n"], 32, st["interp"], *st["push_args"], acc, st["ogrid"], acc_abs=acc_abs,
             acc_count=cnt)
    I = pic.InterpolatorArray(nc, np.float32)
    I.buf.copy_(torch.from_numpy(st["interp"]))
    A = pic.AccumulatorArray(nc, np.float32)
    pic.push(P, I, *st["push_args"], A, None, 8, 8, 8, 1, pic.Boundary.Periodic, exact=True)
    pic.check_status()
    assert np.array_equal(P.download_bytes(), host)
    err = np.abs(A.get().astype(np.float64) - acc)
    assert np.all(err <= reorder_bound(acc_abs, cnt, np.finfo(np.float32).eps))
    # repeated sorts are stable in the key order and keep the population
    sorter(P)
    out = P.download()
    assert np.all(np.diff(out["cell"]) >= 0) and len(out["cell"]) == st["n"]


def test_sort_scratch_too_small_is_rejected():
    import ctypes as C
    from cabanapic_gb300 import capi, pic
    P = pic.ParticleList(1000, np.float32, 32)
    scratch = torch.zeros(1024, dtype=torch.uint8, device="cuda")
    rc = capi.load().raw("cpic_sort_particles")(P.ptr, 1000, 500, 4, 32, scratch.data_ptr(),
                                                scratch.numel(), None)
    assert rc == capi.CPIC_ESCRATCH


@pytest.mark.parametrize("real,vl", [(np.float32, 32), (np.float64, 16)])
def test_out_of_place_sort_matches_in_place(real, vl):
    """cpic_sort_particles_into gathers into a second list in cell order (the
    order within a cell, like the in-place sort's, follows atomic arrival),
    leaving the source untouched; the double-buffered Sorter swaps the list
    onto the sorted buffer."""
    from cabanapic_gb300 import pic
    n = 30011
    st = random_state(nx=9, ny=7, nz=5, n=n, seed=3, real=real, vl=vl)
    A = pic.ParticleList(n, real, vl).upload(st["particles"])
    B = pic.ParticleList(n, real, vl).upload(st["particles"])
    pic.Sorter(A, st["num_cells"])(A)
    s = pic.Sorter(B, st["num_cells"], double_buffer=True)
    before = B.buf
    s(B)
    assert B.buf is not before and s.spare is before
    a, b = A.download(), B.download()
    assert np.array_equal(a["cell"], b["cell"]) and np.all(np.diff(b["cell"]) >= 0)
    ia, ka = _records(a)
    ib, kb = _records(b)
    for x, y in zip(ka, kb):
        assert np.array_equal(x[ia], y[ib])
    assert np.array_equal(s.spare[: B.nbytes].cpu().numpy(), st["particles"].view(np.uint8))


def test_pinned_upload_download_in_pieces():
    """ParticleList.upload_pinned / download_pinned (copies split over side
    streams) move the exact bytes, ordered with the current stream."""
    from cabanapic_gb300 import pic
    n = 100003
    st = random_state(nx=5, ny=5, nz=5, n=n, seed=9)
    pinned = torch.from_numpy(st["particles"].view(np.uint8).copy()).pin_memory()
    P = pic.ParticleList(n, np.float32, 32)
    P.upload_pinned(pinned, pieces=7)
    pic.Sorter(P, st["num_cells"])(P)          # stream-ordered after the upload
    out = torch.empty_like(pinned).pin_memory()
    P.download_pinned(out, pieces=5)
    torch.cuda.current_stream().synchronize()
    assert np.array_equal(out.numpy(), P.download_bytes())
    assert np.all(np.diff(P.download()["cell"]) >= 0)


@pytest.mark.parametrize("kind", ["sorted", "drifted", "random", "out_of_range"])
@pytest.mark.parametrize("real,vl", [(np.float32, 32), (np.float64, 16)])
def test_sort_key_patterns(kind, real, vl):
    """Cell keys as the sort meets them: in cell order (every warp chunk is one
    or two runs of equal keys), a sorted list after some steps of drift (runs
    split by strays), random, and with cells outside [0, num_cells) (sorted
    after every valid cell, in any order among themselves).  The particle
    records are preserved, and the in-place and out-of-place sorts produce
    the same key order."""
    from cabanapic_gb300 import layout as L, pic
    n = 20011
    st = random_state(nx=9, ny=7, nz=5, n=n, seed=11, real=real, vl=vl, sort=kind != "random",
                      disorder=0.2 if kind == "drifted" else 0.0)
    nc = st["num_cells"]
    host = dict(st["host"])
    if kind == "out_of_range":
        rng = np.random.default_rng(3)
        bad = rng.random(n) < 0.05
        host["cell"] = np.where(bad, rng.choice([-7, -1, nc, nc + 3], n), host["cell"]).astype(np.int32)
    packed = L.pack_particles(host, real, vl)
    A = pic.ParticleList(n, real, vl).upload(packed)
    B = pic.ParticleList(n, real, vl).upload(packed)
    pic.Sorter(A, nc)(A)
    pic.Sorter(B, nc, double_buffer=True)(B)
    a, b = A.download(), B.download()
    key = lambda c: np.where((c >= 0) & (c < nc), c, nc)
    assert np.all(np.diff(key(a["cell"])) >= 0)
    assert np.array_equal(key(a["cell"]), key(b["cell"]))
    ia, ka = _records(a)
    ib, kb = _records(b)
    _, k0 = _records(host)
    i0 = np.lexsort(k0[::-1])
    for x, y, z in zip(ka, kb, k0):
        assert np.array_equal(x[ia], y[ib]) and np.array_equal(x[ia], z[i0])


def _ahead_keys(p, steps, cdt, nx, ny, nz, real):
    """Look-ahead keys restated in numpy with the device's operation order:
    the interior cell reached after `steps` pushes of displacement
    2 u cdt / gamma, wrapped periodically; ghost cells keep their index and
    out-of-range cells take the last bucket; the predicted offset is clamped
    to +-(2n - 1).  steps = 0: the cells (a particle on a +face stays in its
    cell)."""
    R = np.dtype(real).type
    sx, sy = nx + 2, ny + 2
    nc = sx * sy * (nz + 2)
    c = p["cell"].astype(np.int64)
    out_of_range = (c < 0) | (c >= nc)
    cc = np.where(out_of_range, 0, c)
    iz = cc // (sx * sy)
    iy = (cc - iz * sx * sy) // sx
    ix = cc - iz * sx * sy - iy * sx
    interior = (ix >= 1) & (ix <= nx) & (iy >= 1) & (iy <= ny) & (iz >= 1) & (iz <= nz)
    ux, uy, uz = p["ux"], p["uy"], p["uz"]
    with np.errstate(all="ignore"):
        rg = R(1) / np.sqrt(R(1) + (ux * ux + (uy * uy + uz * uz)))

        def idx(i, x, u, k, n):
            f = x + R(k) * u * rg
            lim = R(2 * n - 1)
            f = np.where(~(f >= -lim), -lim, f)
            f = np.where(~(f <= lim), lim, f)
            shift = np.floor((f + R(1)) * R(0.5)).astype(np.int64)
            return (i - 1 + shift) % n + 1

        jx = idx(ix, p["x"], ux, 2.0 * steps * cdt[0], nx)
        jy = idx(iy, p["y"], uy, 2.0 * steps * cdt[1], ny)
        jz = idx(iz, p["z"], uz, 2.0 * steps * cdt[2], nz)
    key = np.where(interior, jx + sx * jy + sx * sy * jz, cc) if steps else cc
    return np.where(out_of_range, nc, key)


@pytest.mark.parametrize("real,vl", [(np.float32, 32), (np.float64, 16)])
@pytest.mark.parametrize("steps", [0, 1, 7, 10])
def test_look_ahead_sort_orders_by_predicted_cell(real, vl, steps):
    """cpic_sort_particles_ahead_into: the output is a permutation of the
    input whose look-ahead keys (restated in numpy) are non-decreasing; fast
    particles wrap around the periodic grid several times; ghost and
    out-of-range cells keep their place in the key order.  steps = 0 is the
    cell sort."""
    from cabanapic_gb300 import capi, layout as L, pic
    nx, ny, nz = 9, 7, 5
    n = 30011
    st = random_state(nx=nx, ny=ny, nz=nz, n=n, seed=steps + 3, real=real, vl=vl, crossing=0.4)
    host = {k: v.copy() for k, v in st["host"].items()}
    nc = st["num_cells"]
    host["cell"][:5] = 0                  # a ghost cell
    host["cell"][5:9] = nc + 3           # out of range
    host["ux"][9:12] = np.asarray([np.inf, -np.inf, np.nan], real)
    cdt = (0.45, 0.40, 0.35)
    P = pic.ParticleList(n, real, vl).upload(host)
    srt = pic.Sorter(P, nc, double_buffer=True, steps_ahead=steps, ahead=((nx, ny, nz), cdt)) if steps else \
        pic.Sorter(P, nc, double_buffer=True)
    srt(P)
    out = P.download()
    keys = _ahead_keys(out, steps, cdt, nx, ny, nz, real)
    assert np.all(np.diff(keys) >= 0)
    if steps:
        assert np.any(keys != np.where(out["cell"] >= nc, nc, out["cell"]))  # the keys are not the cells
    ia, ka = _records(host)
    ib, kb = _records(out)
    for x, y in zip(ka, kb):
        assert np.array_equal(x[ia], y[ib])
