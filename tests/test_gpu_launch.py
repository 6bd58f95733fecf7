"""Launch machinery: the CUDA-graph batch (smc_generate_graph) and the
autotuner (smc_autotune).  Both change how the kernels are launched, not
what they compute."""
import numpy as np
import pytest
import torch

from systems import SYSTEMS, values

pytestmark = pytest.mark.gpu


def _bufs(n, dev="cuda"):
    return {"ecc": torch.zeros((n, 49), dtype=torch.float64, device=dev),
            "npart": torch.zeros((n, 2), dtype=torch.int32, device=dev),
            "ncoll": torch.zeros((n,), dtype=torch.int32, device=dev),
            "b": torch.zeros((n,), dtype=torch.float64, device=dev)}


@pytest.mark.parametrize("tensor_cores", [True, False])
def test_graph_replays_equal_eager_batches(tensor_cores):
    from supermc_gb300.engine import Engine
    vals = values(SYSTEMS["pbpb2760"], ecc_from_order=2, ecc_to_order=5)
    eng = Engine(dict(vals), seed=4)
    eng.set_grid_path(tensor_cores)
    n = 5000                                # two chunks, the second partial
    g, e = _bufs(n), _bufs(n)
    for first in (0, 7000, 123456):         # capture (eager), then two replays
        eng.generate_graph_into(first, n, g)
        eng.generate_into(first, n, e)
        torch.cuda.synchronize()
        for k in g:
            assert torch.equal(g[k], e[k]), (first, k)
    st = eng.stats()
    assert st["launches"] > 0


def test_graph_recaptures_for_new_sizes():
    from supermc_gb300.engine import Engine
    eng = Engine(dict(values(SYSTEMS["auau200"])), seed=5)
    for n in (100, 300, 100):
        g, e = _bufs(n), _bufs(n)
        eng.generate_graph_into(11, n, g)
        eng.generate_graph_into(11, n, g)   # a replay
        eng.generate_into(11, n, e)
        torch.cuda.synchronize()
        assert torch.equal(g["ecc"], e["ecc"]) and torch.equal(g["ncoll"], e["ncoll"])


def test_autotune_keeps_results():
    from supermc_gb300.engine import Engine
    eng = Engine(dict(values(SYSTEMS["pbpb2760"], ecc_from_order=2, ecc_to_order=5)), seed=6)
    before = eng.generate(0, 64, want=("ecc", "npart", "ncoll"))
    t = eng.autotune(2048)
    assert t["chunk"] in (2048, 4096, 8192, 16384)
    rates = [v for v in t["events_per_s"].values() if v > 0]
    assert len(rates) >= 4 and max(rates) == t["events_per_s"][
        f"{'tensor_cores' if t['tensor_cores'] else 'cuda_cores'}_{t['chunk']}"]
    after = eng.generate(0, 64, want=("ecc", "npart", "ncoll"))
    np.testing.assert_array_equal(before["npart"], after["npart"])
    np.testing.assert_array_equal(before["ncoll"], after["ncoll"])
    # the two splat paths agree within FP32 rounding (eps within 1e-6, the
    # integral of column 47 to 1e-6 relative)
    cols = [k for k in range(45) if k % 5 != 4]
    np.testing.assert_allclose(after["ecc"][:, cols], before["ecc"][:, cols], rtol=0, atol=1e-6)
    np.testing.assert_allclose(after["ecc"][:, 45:], before["ecc"][:, 45:], rtol=1e-6)
