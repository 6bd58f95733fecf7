"""Mixed-system batches through the C ABI (smc_generate_mixed): every event of
the batch equals the same event (seed, event id) generated by a context of its
own system alone -- the per-event Philox streams do not depend on the batch."""
import numpy as np
import pytest

from systems import BASE, values
from test_gpu_parity import engine

pytestmark = pytest.mark.gpu

# p+Pb, d+Au (Hulthen deuteron), Cu+Cu, deformed U+U, Au+Au with the
# Woods-Saxon parameters and hard core of the mixed workload
MIXED = [
    dict(Aproj=1, Atarg=208, ecm=5020),
    dict(Aproj=2, Atarg=197, ecm=200),
    dict(Aproj=63, Atarg=63, ecm=200, proj_R=4.2, proj_a=0.596, targ_R=4.2, targ_a=0.596),
    dict(Aproj=238, Atarg=238, ecm=200, proj_deformed=1, targ_deformed=1, proj_R=6.81, proj_a=0.55,
         targ_R=6.81, targ_a=0.55),
    dict(Aproj=197, Atarg=197, ecm=200, proj_R=6.38, proj_a=0.535, targ_R=6.38, targ_a=0.535,
         proj_d_min=0.4, targ_d_min=0.4),
]


@pytest.mark.parametrize("tensor_cores", [True, False])
def test_mixed_batch_equals_single_system_runs(tensor_cores):
    base = values(dict(BASE, **MIXED[-1]))
    n = 5 * 24
    sel = np.random.default_rng(3).permutation(np.arange(n) % len(MIXED)).astype(np.int32)
    eng = engine(base, seed=17)
    eng.set_grid_path(tensor_cores)
    want = ("ecc", "npart", "ncoll", "b", "attempts")
    mixed = eng.generate_mixed(MIXED, sel, first_event=1000, want=want)
    for k, sysv in enumerate(MIXED):
        single = engine(values(dict(BASE, **sysv)), seed=17)
        single.set_grid_path(tensor_cores)
        ref = single.generate(1000, n, want=want)
        idx = np.flatnonzero(sel == k)
        for key in want:
            np.testing.assert_array_equal(mixed[key][idx], ref[key][idx], err_msg=f"system {k} {key}")
    # the systems are what they claim: participants within each system's size
    npart = mixed["npart"].sum(axis=1)
    assert npart[sel == 0].max() <= 1 + 208 and (mixed["npart"][sel == 0, 0] == 1).all()
    assert (mixed["npart"][sel == 1, 0] <= 2).all()
    assert npart[sel == 3].max() > npart[sel == 2].max()


def test_mixed_batch_rejects_incompatible_systems():
    from supermc_gb300._lib import SmcError
    eng = engine(values(dict(BASE, **MIXED[-1])), seed=1)
    with pytest.raises(SmcError):   # a different grid spacing
        eng.generate_mixed([dict(MIXED[0], dx=0.2)], np.zeros(4, np.int32))
    with pytest.raises(SmcError):   # system index out of range
        eng.generate_mixed(MIXED[:2], np.array([0, 1, 2], np.int32))


@pytest.mark.parametrize("tensor_cores", [False, True])
def test_mixed_graph_replays_equal_eager_batches(tensor_cores):
    """smc_generate_mixed_graph: the first call runs eagerly and captures the
    batch; replays with new event ids equal smc_generate_mixed on those ids.
    An eager call that grows the context's buffers in between makes the next
    call capture again (the old graph's buffers are gone)."""
    import torch
    base = values(dict(BASE, **MIXED[-1]), ecc_from_order=2, ecc_to_order=5)
    n = 5 * 40
    sel = np.random.default_rng(8).permutation(np.arange(n) % len(MIXED)).astype(np.int32)
    eng = engine(base, seed=23)
    eng.set_grid_path(tensor_cores)
    dev = torch.device("cuda", 0)

    def bufs():
        return {"ecc": torch.zeros((n, 49), dtype=torch.float64, device=dev),
                "npart": torch.zeros((n, 2), dtype=torch.int32, device=dev),
                "ncoll": torch.zeros((n,), dtype=torch.int32, device=dev)}
    g = bufs()
    for first in (0, 5000, 9000):
        eng.generate_mixed(MIXED, sel, first_event=first, device_bufs=g, graph=True)
        ref = eng.generate_mixed(MIXED, sel, first_event=first, want=("ecc", "npart", "ncoll"))
        for key in ("ecc", "npart", "ncoll"):
            np.testing.assert_array_equal(g[key].cpu().numpy(), ref[key], err_msg=f"{first} {key}")
        if first == 5000:
            eng.generate(0, 4 * n)   # grows the context's buffers
