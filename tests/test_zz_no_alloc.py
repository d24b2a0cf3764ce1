"""nlc_linenergies_noalloc against nlc_linenergies and the oracle, through the C ABI.

The allocation-free entry point serves callers that may not allocate device memory when they ask
for the diagnostics (an application whose device memory is owned by its own pool, or a service that
reserves all of it at start-up).  It keeps its temporaries in one static device array shared by
every call, so each case calls it twice in a row on different data and checks every result against
the regular entry point (which allocates through its plan) and against the oracle, within the
diagnostics tolerance of the other tests (1e-10).  The cases include lengths with odd prime
factors up to the entry point's limit of 61 and an entropy mask.  This file is named to be
collected last.
"""
import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu

TOL = 1e-10

CASES = [
    ("FPUT", 64, dict(alpha=0.0, beta=1.0), 0.0),
    ("DNKG", 128, dict(m=1.0, beta=1.0), 1.0),
    ("Toda", 100, dict(alpha=0.5), 0.0),
    ("DNLS", 1024, dict(beta=1.0), 0.0),
    ("DNKG", 2048, dict(m=0.3, beta=0.5), 0.3),
    ("FPUT", 61, dict(alpha=0.25, beta=1.0), 0.0),     # the largest prime accepted
    ("DNLS", 118, dict(beta=1.0), 0.0),                 # 2 x 59
    ("DNKG", 3 * 5 * 7 * 11, dict(m=0.7, beta=1.0), 0.7),
]


def _mask(n, masked):
    if not masked:
        return None
    mask = np.zeros(n, dtype=np.uint8)
    mask[1:min(n, 9)] = 1   # a few low modes
    return mask


@pytest.mark.parametrize("masked", [False, True], ids=["all-modes", "masked"])
@pytest.mark.parametrize("case", CASES, ids=lambda c: f"{c[0]}-{c[1]}")
def test_noalloc_matches_regular_entry_point_twice(gpu, case, masked):
    torch = pytest.importorskip("torch")
    model, n, params, m = case
    copies = 333
    rng = np.random.default_rng(n)
    mask = _mask(n, masked)
    plan = gpu.Plan(gpu.Model(model, n, copies, 0.05, entropy_mask=mask, **params))
    mdl = O.Model(model, n, copies, 0.05, **params)
    stream = torch.cuda.current_stream().cuda_stream
    mask_dev = torch.from_numpy(mask).cuda() if mask is not None else None
    for call in range(2):
        host = rng.standard_normal((copies, n, 2)) * (1 + call)
        state = torch.from_numpy(host).cuda()
        lin_ref = torch.zeros(n, dtype=torch.float64, device="cuda")
        ent_ref = torch.zeros(2, dtype=torch.float64, device="cuda")
        plan.linenergies(state.data_ptr(), lin_ref.data_ptr(), ent_ref.data_ptr(), stream)
        lin = torch.full((n,), float("nan"), dtype=torch.float64, device="cuda")
        ent = torch.full((2,), float("nan"), dtype=torch.float64, device="cuda")
        gpu.linenergies_noalloc(model, n, copies, m, state.data_ptr(), lin.data_ptr(), ent.data_ptr(),
                                mask_dev.data_ptr() if mask_dev is not None else 0, stream)
        torch.cuda.synchronize()
        a, b = lin.cpu().numpy(), lin_ref.cpu().numpy()
        assert np.abs(a - b).max() <= TOL * np.abs(b).max(), f"call {call}: linenergies differ from nlc_linenergies"
        ea, eb = ent.cpu().numpy(), ent_ref.cpu().numpy()
        assert np.all(np.abs(ea - eb) <= TOL * np.maximum(1.0, np.abs(eb))), f"call {call}: entropies differ"
        exp = O.linenergies(mdl, host)
        assert np.abs(a - exp).max() <= TOL * np.abs(exp).max(), f"call {call}: linenergies differ from the oracle"
        ewt, einf = O.entropies(exp, O.a0is0(mdl), mask)
        assert abs(ea[0] - ewt) <= TOL * max(1.0, abs(ewt)) and abs(ea[1] - einf) <= TOL * max(1.0, abs(einf))


def test_noalloc_rejects_oversized_chains(gpu):
    with pytest.raises(gpu.NlcError) as e:
        gpu.linenergies_noalloc("FPUT", 8192, 4, 0.0, 1, 1)
    assert e.value.code == gpu.EINVAL and "4096" in str(e.value)


def test_noalloc_rejects_large_prime_factors(gpu):
    with pytest.raises(gpu.NlcError) as e:
        gpu.linenergies_noalloc("DNKG", 4093, 4, 1.0, 1, 1)
    assert e.value.code == gpu.EUNSUPPORTED and "prime factor above 61" in str(e.value)
