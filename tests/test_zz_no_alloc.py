"""nlc_linenergies_noalloc against nlc_linenergies, through the C ABI.

The allocation-free entry point serves callers that may not allocate device memory when they ask
for the diagnostics (for example while a CUDA graph is being recorded, or inside an application
whose device memory is owned by its own pool).  It keeps its temporaries in one static device
array shared by every call, so this test calls it twice in a row on different data and checks each
result against the regular entry point (which allocates through its plan), within the diagnostics
tolerance of the other tests (1e-10).  This file is named to be collected last.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-10

CASES = [
    ("FPUT", 64, dict(alpha=0.0, beta=1.0), 0.0),
    ("DNKG", 128, dict(m=1.0, beta=1.0), 1.0),
    ("Toda", 100, dict(alpha=0.5), 0.0),
    ("DNLS", 1024, dict(beta=1.0), 0.0),
    ("DNKG", 2048, dict(m=0.3, beta=0.5), 0.3),
]


@pytest.mark.parametrize("case", CASES, ids=lambda c: f"{c[0]}-{c[1]}")
def test_noalloc_matches_regular_entry_point_twice(gpu, case):
    torch = pytest.importorskip("torch")
    model, n, params, m = case
    copies = 333
    rng = np.random.default_rng(n)
    plan = gpu.Plan(gpu.Model(model, n, copies, 0.05, **params))
    stream = torch.cuda.current_stream().cuda_stream
    for call in range(2):
        state = torch.from_numpy(rng.standard_normal((copies, n, 2)) * (1 + call)).cuda()
        lin_ref = torch.zeros(n, dtype=torch.float64, device="cuda")
        ent_ref = torch.zeros(2, dtype=torch.float64, device="cuda")
        plan.linenergies(state.data_ptr(), lin_ref.data_ptr(), ent_ref.data_ptr(), stream)
        lin = torch.full((n,), float("nan"), dtype=torch.float64, device="cuda")
        ent = torch.full((2,), float("nan"), dtype=torch.float64, device="cuda")
        gpu.linenergies_noalloc(model, n, copies, m, state.data_ptr(), lin.data_ptr(), ent.data_ptr(), 0, stream)
        torch.cuda.synchronize()
        a, b = lin.cpu().numpy(), lin_ref.cpu().numpy()
        assert np.abs(a - b).max() <= TOL * np.abs(b).max(), f"call {call}: linenergies differ"
        ea, eb = ent.cpu().numpy(), ent_ref.cpu().numpy()
        assert np.all(np.abs(ea - eb) <= TOL * np.maximum(1.0, np.abs(eb))), f"call {call}: entropies differ"


def test_noalloc_rejects_oversized_chains(gpu):
    with pytest.raises(gpu.NlcError) as e:
        gpu.linenergies_noalloc("FPUT", 8192, 4, 0.0, 1, 1)
    assert e.value.code == gpu.EINVAL and "4096" in str(e.value)
