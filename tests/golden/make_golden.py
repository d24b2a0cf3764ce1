"""Writes the golden fixtures of this directory from the oracle (the C restatement of the reference's
algorithm, oracle/nlc_oracle.c) on seeded inputs.  Run from the repository root after building the
oracle:  python tests/golden/make_golden.py

Each fixture <model>_n<n>.npz holds the input state (reference -i layout, [copies][n][2]), the model
parameters, the state after `steps` steps of `batching` in the engine's operation order (the GPU
integrators must reproduce it bit for bit) and in the reference CPU operation order, and the linear
energies and {WT, INF} entropies of the device-order result.  The reference itself ships no golden
vectors or tests (it cannot be built here either), so these pin the oracle: test_golden.py checks the
oracle of the machine the tests run on against them (an x86 and an Arm build must agree), and the GPU
tests check the engine against them.
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

import oracle as O  # noqa: E402

HERE = os.path.dirname(os.path.abspath(__file__))

# (model, n, copies, dt, params, steps, batching); DNLS n = 39 has the prime factor 13 (the
# engine's padded-convolution form), n = 12 is smooth
CASES = [
    ("DNKG", 16, 3, 0.05, dict(m=1.0, beta=1.0), 20, 10),
    ("DNKG", 37, 3, 0.05, dict(m=0.5, beta=0.7), 20, 10),
    ("FPUT", 16, 3, 0.1, dict(alpha=0.0, beta=1.0), 20, 10),
    ("FPUT", 37, 3, 0.05, dict(alpha=0.3, beta=0.8), 20, 10),
    ("Toda", 16, 3, 0.05, dict(alpha=0.5), 20, 10),
    ("Toda", 37, 3, 0.05, dict(alpha=0.8), 20, 10),
    ("dDNKG", 16, 3, 0.05, dict(beta=1.0), 20, 10),
    ("DNLS", 12, 2, 0.01, dict(beta=1.0), 10, 5),
    ("DNLS", 39, 2, 0.01, dict(beta=1.0), 10, 5),
]


def case_name(model, n):
    return f"{model}_n{n}.npz"


def make(model, n, copies, dt, params, steps, batching):
    rng = np.random.default_rng(1000 + n + 7 * len(model))
    state = 0.4 * rng.standard_normal((copies, n, 2))
    masses = rng.uniform(1.0, 3.0, n) if model == "dDNKG" else None
    mdl = O.Model(model, n, copies, dt, masses=masses, **params)
    out = {"model": model, "n": n, "copies": copies, "dt": dt, "steps": steps, "batching": batching,
           "state_in": state, "masses": masses if masses is not None else np.zeros(0),
           "m": params.get("m", 0.0), "alpha": params.get("alpha", 0.0), "beta": params.get("beta", 0.0)}
    dev = O.advance(mdl, state, steps, batching, order=O.ORDER_DEVICE).reshape(copies, n, 2)
    out["state_device_order"] = dev
    if model != "DNLS":
        out["state_reference_order"] = O.advance(mdl, state, steps, batching,
                                                 order=O.ORDER_REFERENCE).reshape(copies, n, 2)
    lin = O.linenergies(mdl, dev)
    out["linenergies"] = lin
    out["entropies"] = np.array(O.entropies(lin, O.a0is0(mdl)))
    return out


def main():
    for case in CASES:
        d = make(*case)
        np.savez(os.path.join(HERE, case_name(case[0], case[1])), **d)
        print("wrote", case_name(case[0], case[1]))


if __name__ == "__main__":
    main()
