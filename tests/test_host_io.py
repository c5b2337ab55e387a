"""The host I/O step (wrfgpu_bind_host_state / wrfgpu_step_host): the state
of a host time loop that copies the prognostic fields in, steps and copies
them out every step, with the copies captured in the step's graph (the
passive scalars' uploads during stage 1's dynamics, the dry state's
download during the last stage's scalar transport, the passive scalars'
downloads during the next step of the same call), equals the per-field
set / step / get loop bit for bit."""
import numpy as np
import pytest

from wrf_gb300 import abi, cases
from wrf_gb300 import gpu as G

pytestmark = pytest.mark.gpu

DRY = ("u_2", "v_2", "w_2", "t_2", "ph_2", "mu_2", "p", "al")


def _pinned(n):
    import torch
    return torch.empty(n, dtype=torch.float32, pin_memory=True).numpy()


def _fids(case):
    nsp = case.desc.n_moist + case.desc.n_scalar
    return [abi.FIELD_ID[nm] for nm in DRY] + [abi.species_id(s) for s in range(nsp)]


@pytest.mark.parametrize("flags", [0, G.FLAG_NO_GRAPH], ids=["graph", "direct"])
def test_step_host_equals_set_step_get(gpulib, flags):
    """Three large steps (an odd number of species-buffer swaps per step, so
    the bound species alternate buffers between graph launches) of a case
    with qv and three passive scalars: every bound field after each step
    bit for bit the per-field loop's."""
    case = cases.small_case(nx=40, ny=20, kde=16, n_scalar=3, seed=8)
    ref = G.Domain(case, flags)
    dut = G.Domain(case, flags)
    fids = _fids(case)
    host_ref = {f: np.array(ref.get(0, f), dtype=np.float32).ravel() for f in fids}
    bufs = []
    for f in fids:
        b = _pinned(host_ref[f].size)
        b[:] = host_ref[f]
        bufs.append(b)
    dut.bind_host_state(0, fids, bufs)
    for step in range(3):
        for f in fids:
            ref.set(0, f, host_ref[f])
        ref.step(1)
        ref.sync()
        for f in fids:
            host_ref[f] = np.array(ref.get(0, f), dtype=np.float32).ravel()
        dut.step_host(1)
        bad = [f for f, b in zip(fids, bufs) if not np.array_equal(b, host_ref[f])]
        assert not bad, (step, bad)
    # one call of three steps: the passive scalars' downloads of steps 1 and
    # 2 cross the link during the next step, the last at the end of the call
    dut.step_host(3)
    for step in range(3):
        for f in fids:
            ref.set(0, f, host_ref[f])
        ref.step(1)
        ref.sync()
        for f in fids:
            host_ref[f] = np.array(ref.get(0, f), dtype=np.float32).ravel()
    bad = [f for f, b in zip(fids, bufs) if not np.array_equal(b, host_ref[f])]
    assert not bad, bad
    # the device state also agrees (the spare species buffers included)
    dut.step(1)
    ref.step(1)
    dut.sync(); ref.sync()
    for f in fids:
        assert np.array_equal(dut.get(0, f), ref.get(0, f)), f
    dut.unbind_host_state()


@pytest.mark.parametrize("lateral", ["periodic", "open"])
def test_step_host_many_passive_scalars(gpulib, lateral):
    """qv and six passive scalars: stage 1's transport of a host I/O step
    runs in two launches (the pairs whose scalars are across first, the
    last pair after every upload); one call of three steps and then one
    step per call give the per-field loop's bits, on a periodic domain and
    on one open on all four sides (the edge strips run before the species'
    end-of-step fill that a call's earlier steps issue early)."""
    case = cases.small_case(nx=36, ny=20, kde=14, n_scalar=6, seed=21)
    if lateral == "open":
        case = cases.open_boundaries(case)
    ref = G.Domain(case)
    dut = G.Domain(case)
    fids = _fids(case)
    host_ref = {f: np.array(ref.get(0, f), dtype=np.float32).ravel() for f in fids}
    bufs = []
    for f in fids:
        b = _pinned(host_ref[f].size)
        b[:] = host_ref[f]
        bufs.append(b)
    dut.bind_host_state(0, fids, bufs)
    for calls in ([3], [1, 1]):
        for n in calls:
            dut.step_host(n)
            for _ in range(n):
                for f in fids:
                    ref.set(0, f, host_ref[f])
                ref.step(1)
                ref.sync()
                for f in fids:
                    host_ref[f] = np.array(ref.get(0, f), dtype=np.float32).ravel()
            bad = [f for f, b in zip(fids, bufs) if not np.array_equal(b, host_ref[f])]
            assert not bad, (calls, bad)
    dut.unbind_host_state()


def test_step_host_separate_in_out_and_refusals(gpulib):
    """Inputs and outputs in different buffers (the inputs are not written),
    an output-only field, and the refusals: pageable memory, a wrong count,
    an unknown field, a step with nothing bound."""
    case = cases.small_case(nx=20, ny=12, kde=14, n_scalar=1, seed=4)
    dom = G.Domain(case)
    fids = _fids(case)
    ins, outs = [], []
    for f in fids:
        a = np.array(dom.get(0, f), dtype=np.float32).ravel()
        b = _pinned(a.size); b[:] = a
        o = _pinned(a.size); o[:] = np.nan
        ins.append(b); outs.append(o)
    with pytest.raises(G.WrfGpuError):
        dom.step_host(1)
    keep = [x.copy() for x in ins]
    dom.bind_host_state(0, fids, ins, outs)
    w1 = _pinned(dom.field_size(0, abi.FIELD_ID["ww"]))
    dom.bind_host_state(0, [abi.FIELD_ID["ww"]], [None], [w1])
    dom.step_host(1)
    assert all(np.array_equal(a, b) for a, b in zip(ins, keep))
    assert all(np.isfinite(o).all() for o in outs)
    assert np.isfinite(w1).all()
    ref = G.Domain(case)
    ref.step(1)
    ref.sync()
    for f, o in zip(fids, outs):
        assert np.array_equal(o, np.asarray(ref.get(0, f), dtype=np.float32).ravel()), f
    # one call of three steps: every step starts again from the unchanged
    # inputs (the next step's inputs cross behind this step's downloads,
    # each after the download that frees its staging buffer)
    for o in outs:
        o[:] = np.nan
    dom.step_host(3)
    assert all(np.array_equal(a, b) for a, b in zip(ins, keep))
    for f, o in zip(fids, outs):
        assert np.array_equal(o, np.asarray(ref.get(0, f), dtype=np.float32).ravel()), f
    pageable = np.zeros(dom.field_size(0, fids[0]), np.float32)
    with pytest.raises(G.WrfGpuError):
        dom.bind_host_state(0, [fids[0]], [pageable])
    with pytest.raises(G.WrfGpuError):
        dom.bind_host_state(0, [fids[0]], [_pinned(10)])
    with pytest.raises(G.WrfGpuError):
        dom.bind_host_state(0, [9999], [_pinned(10)])


def test_step_host_two_members_of_an_ensemble(gpulib):
    """Both members of an uneven two-member ensemble bound (their fields
    interleaved in the binding order): each member's outputs after two
    steps of one call equal its own plain loop's."""
    members = [cases.small_case(nx=24, ny=12, kde=14, n_scalar=2, seed=12),
               cases.small_case(nx=16, ny=20, kde=18, n_scalar=1, seed=13)]
    ens = G.Ensemble.from_cases(members)
    bufs = {}
    for m, cs in enumerate(members):
        for f in _fids(cs):
            b = _pinned(ens.field_size(m, f))
            b[:] = np.asarray(ens.get(m, f), dtype=np.float32)
            bufs[(m, f)] = b
    for m, cs in enumerate(members):
        fids = _fids(cs)
        ens.bind_host_state(m, fids, [bufs[(m, f)] for f in fids])
    ens.step_host(2)
    for m, cs in enumerate(members):
        ref = G.Domain(cs)
        ref.step(2)
        ref.sync()
        for f in _fids(cs):
            assert np.array_equal(bufs[(m, f)], np.asarray(ref.get(0, f), dtype=np.float32)), (m, f)
