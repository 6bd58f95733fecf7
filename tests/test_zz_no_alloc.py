"""smc_inject_noalloc, the entry point for callers that cannot allocate
device memory, against the regular injected-positions entry point.

Both run the same pipeline; the no-allocation variant keeps its
intermediate data in a fixed static device array instead of context
buffers.  Two calls in a row with different events check that the shared
array carries nothing over from one call to the next.  Collected last on
purpose (file name) so a stop-at-first-failure run has already run the rest.
"""
import ctypes

import numpy as np
import pytest

from systems import SYSTEMS, oracle_params, values

pytestmark = pytest.mark.gpu

ECC_ATOL = 1e-6
GRID_RTOL = 2e-5


def _positions(oracle, vals, n, seed):
    ev = oracle.event(oracle_params(vals))
    nA, nB = oracle.nucleus(int(vals["aproj"])), oracle.nucleus(int(vals["atarg"]))
    rng = np.random.default_rng(seed)
    pa, pb, bs = [], [], []
    k = 0
    while len(bs) < n:
        b = float(rng.uniform(0, 14))
        ev.populate_philox(nA, nB, b, seed, k, 0)
        k += 1
        if ev.pair() == 0:
            continue
        pa.append(ev.nucleons(0)[:, :2]); pb.append(ev.nucleons(1)[:, :2]); bs.append(b)
    return np.array(pa), np.array(pb), np.array(bs)


def _noalloc(lib, params, pa, pb, bs, n, nx, ny):
    import torch
    dev = torch.device("cuda", 0)
    d_pa = torch.tensor(pa, device=dev)
    d_pb = torch.tensor(pb, device=dev)
    d_b = torch.tensor(bs, device=dev)
    d_ecc = torch.full((n, 49), float("nan"), dtype=torch.float64, device=dev)
    d_rho = torch.full((n, nx, ny), float("nan"), dtype=torch.float32, device=dev)
    d_st = torch.full((n,), -1, dtype=torch.int32, device=dev)
    torch.cuda.synchronize()
    # the call allocates nothing: the device's free memory and torch's
    # allocator are where they were
    free0 = torch.cuda.mem_get_info()[0]
    alloc0 = torch.cuda.memory_allocated()
    st = lib.smc_inject_noalloc(ctypes.byref(params), n, d_pa.data_ptr(), d_pb.data_ptr(), d_b.data_ptr(),
                                d_ecc.data_ptr(), d_rho.data_ptr(), d_st.data_ptr(), None)
    torch.cuda.synchronize()
    moved = (torch.cuda.mem_get_info()[0] != free0, torch.cuda.memory_allocated() != alloc0)
    return st, d_ecc.cpu().numpy(), d_rho.cpu().numpy(), d_st.cpu().numpy(), moved


@pytest.mark.parametrize("over", [dict(), dict(which_mc_model=7), dict(cc_fluctuation_model=6)],
                         ids=["glauber", "sqrt_ta_tb", "gamma_weights"])
def test_noalloc_matches_context_entry_point(oracle, over):
    from supermc_gb300 import _lib
    from supermc_gb300.engine import Engine
    vals = values(SYSTEMS["auau200"], **over)
    eng = Engine(vals, seed=0)
    lib = _lib.load()
    n = 12
    for call, seed in enumerate((101, 202)):
        pa, pb, bs = _positions(oracle, values(SYSTEMS["auau200"]), n, seed)
        ref = eng.inject(pa, pb, bs, want=("ecc", "rho"))
        st, ecc, rho, status, moved = _noalloc(lib, eng.params, pa, pb, bs, n, eng.nx, eng.ny)
        assert st == 0, f"call {call}: status {st}"
        assert (status == 0).all()
        if call == 1:   # the first call on the device may load the module
            assert moved == (False, False), moved
        eps_cols = [5 * k + c for k in range(9) for c in range(4)]
        np.testing.assert_allclose(ecc[:, eps_cols], ref["ecc"][:, eps_cols], rtol=0, atol=ECC_ATOL)
        np.testing.assert_allclose(ecc[:, 45:], ref["ecc"][:, 45:], rtol=1e-6)
        for k in range(n):
            assert np.abs(rho[k] - ref["rho"][k]).max() <= GRID_RTOL * ref["rho"][k].max()


def test_noalloc_reports_collision_capacity(oracle):
    """An event with more binary collisions than max_collisions gets
    SMC_ERR_CAPACITY (6) in its status entry, the others are unaffected."""
    from supermc_gb300 import _lib
    from supermc_gb300.engine import smc_params_from
    vals = values(SYSTEMS["pbpb2760"], max_collisions=300)
    p = smc_params_from(vals)
    ev = oracle.event(oracle_params(values(SYSTEMS["pbpb2760"])))
    nuc = oracle.nucleus(208)
    pa, pb, bs, nc = [], [], [], []
    for k, b in enumerate((0.5, 11.0)):   # a head-on and a peripheral event
        ev.populate_philox(nuc, nuc, b, 5, k, 0)
        pa.append(ev.nucleons(0)[:, :2]); pb.append(ev.nucleons(1)[:, :2]); bs.append(b)
        ev.inject(pa[-1], pb[-1])
        nc.append(ev.pair())
    assert nc[0] > 300 and 0 < nc[1] <= 300
    lib = _lib.load()
    nx = ny = 261
    st, ecc, rho, status, _ = _noalloc(lib, p, np.array(pa), np.array(pb), np.array(bs), 2, nx, ny)
    assert st == 0
    assert status[0] == 6 and status[1] == 0


def test_noalloc_refuses_oversized_request():
    from supermc_gb300 import _lib
    from supermc_gb300.engine import smc_params_from
    vals = values(SYSTEMS["pbpb2760"])
    p = smc_params_from(vals)
    lib = _lib.load()
    # the sizes are checked before any pointer is used
    fake = 256
    st = lib.smc_inject_noalloc(ctypes.byref(p), 100000, fake, fake, None, fake, fake, fake, None)
    assert st == 9   # SMC_ERR_SCRATCH_LIMIT
