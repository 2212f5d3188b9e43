"""Failure detection on the device: bad inputs made on the host must come back
as status bits, without faulting the GPU, and leave the other particles
pushed correctly."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from support import random_state  # noqa: E402

pytestmark = pytest.mark.gpu


def _setup(st):
    from cabanapic_gb300 import pic
    nc = st["num_cells"]
    P = pic.ParticleList(st["n"], np.float32, 32).upload(st["particles"])
    I = pic.InterpolatorArray(nc, np.float32)
    I.buf.copy_(torch.from_numpy(st["interp"]))
    A = pic.AccumulatorArray(nc, np.float32)
    return P, I, A


def test_cell_out_of_range_is_reported_and_skipped(orc):
    from cabanapic_gb300 import capi, layout as L, pic
    st = random_state(n=2000, seed=12)
    host = dict(st["host"])
    host["cell"] = host["cell"].copy()
    host["cell"][[5, 700]] = [-3, st["num_cells"] + 10]
    st["particles"] = L.pack_particles(host, np.float32, 32)
    P, I, A = _setup(st)
    pic.push(P, I, *st["push_args"], A, None, st["nx"], st["ny"], st["nz"], 1, pic.Boundary.Periodic)
    with pytest.raises(capi.CpicDeviceError) as ei:
        pic.check_status()
    assert ei.value.bits & capi.CPIC_STATUS_CELL_RANGE
    out = P.download()
    # the two bad particles are left untouched
    for k in ("x", "y", "z", "ux", "uy", "uz", "cell"):
        assert np.array_equal(out[k][[5, 700]], host[k][[5, 700]])
    # the status was cleared by check_status; a clean push reports nothing
    good = random_state(n=500, seed=13)
    P2, I2, A2 = _setup(good)
    pic.push(P2, I2, *good["push_args"], A2, None, good["nx"], good["ny"], good["nz"], 1,
             pic.Boundary.Periodic)
    pic.check_status()


def test_nonfinite_momentum_is_reported(orc):
    from cabanapic_gb300 import capi, layout as L, pic
    st = random_state(n=1000, seed=14)
    host = dict(st["host"])
    host["ux"] = host["ux"].copy()
    host["ux"][17] = np.nan
    st["particles"] = L.pack_particles(host, np.float32, 32)
    P, I, A = _setup(st)
    pic.push(P, I, *st["push_args"], A, None, st["nx"], st["ny"], st["nz"], 1, pic.Boundary.Periodic,
             exact=True)
    with pytest.raises(capi.CpicDeviceError) as ei:
        pic.check_status()
    assert ei.value.bits & capi.CPIC_STATUS_NONFINITE
    # the reference's own behaviour for the NaN particle (one NaN streak, then stop)
    ref = st["particles"].copy()
    acc = np.zeros((st["num_cells"], 3, 4), np.float32)
    orc.push(ref, st["n"], 32, st["interp"], *st["push_args"], acc, st["ogrid"])
    got = P.download()
    want = L.unpack_particles(ref, st["n"], np.float32, 32)
    keep = np.arange(st["n"]) != 17   # NaN payload bits differ between CPU and GPU
    for k in ("x", "y", "z", "ux", "uy", "uz", "cell"):
        assert np.array_equal(got[k][keep], want[k][keep])
    for k in ("x", "y", "z", "ux", "uy", "uz"):
        assert np.isnan(got[k][17]) and np.isnan(want[k][17])
    assert got["cell"][17] == want["cell"][17]


def test_reflect_boundary_rejected():
    from cabanapic_gb300 import capi, pic
    st = random_state(n=64, seed=15)
    P, I, A = _setup(st)
    with pytest.raises(capi.CpicError) as ei:
        pic.push(P, I, *st["push_args"], A, None, st["nx"], st["ny"], st["nz"], 1, pic.Boundary.Reflect)
    assert ei.value.code == capi.CPIC_EUNSUPPORTED


def test_bounded_wait_gives_up_and_reports_the_pipeline_bit(orc):
    """The tiled push's mbarrier wait, run on a barrier phase that nothing
    completes, gives up after its cycle limit (here ~2^22 cycles, a few ms)
    and sets CPIC_STATUS_PIPELINE; the context stays usable and the next
    push is still exact."""
    import time
    from cabanapic_gb300 import capi, pic
    status = pic.status_word()
    pic.check_status()  # start clean
    t0 = time.perf_counter()
    capi.load().call("cpic_selftest_bounded_wait", 1 << 22, status.data_ptr(),
                     torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    assert time.perf_counter() - t0 < 5.0
    with pytest.raises(capi.CpicDeviceError) as ei:
        pic.check_status()
    assert ei.value.bits == capi.CPIC_STATUS_PIPELINE
    assert capi.load().raw("cpic_selftest_bounded_wait")(1 << 40, status.data_ptr(), None) == capi.CPIC_EINVAL
    # the device still works: an exact push matches the oracle bit for bit
    st = random_state(n=3000, seed=14)
    P, I, A = _setup(st)
    host = st["particles"].copy()
    acc = np.zeros((st["num_cells"], 3, 4), np.float32)
    orc.push(host, st["n"], 32, st["interp"], *st["push_args"], acc, st["ogrid"])
    pic.push(P, I, *st["push_args"], A, None, st["nx"], st["ny"], st["nz"], 1, pic.Boundary.Periodic, exact=True)
    pic.check_status()
    assert np.array_equal(P.download_bytes(), host)
