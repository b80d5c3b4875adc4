"""Writes the golden fixtures used by the parity tests.

Run from the repository root:  python tests/golden/make_golden.py

* index_streams.npz -- minibatch index streams produced by the reference
  loader's own call (numpy Generator.choice(arange(N), n, replace=True) on
  default_rng(SeedSequence(seed).spawn(1)[0]), jax_sgmc/data/numpy_loader.py:
  261-265,382-389) for seeds 0..7, N in {10^4, 10^6}, n in {128, 1024}, three
  consecutive minibatches each, with the PCG64 state before and after.
* philox_kat.json -- Philox4x32-10 known-answer vectors (Random123).
* potential_kat.json -- closed-form potentials of tests/test_potential.py
  (lines 66-122) for obs in {7, 11}, dim in {3, 5}.
"""

import json
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent


def pcg_words(state):
  st, inc = state["state"]["state"], state["state"]["inc"]
  m = (1 << 64) - 1
  return np.array([(st >> 64) & m, st & m, (inc >> 64) & m, inc & m,
                   int(state["has_uint32"]), int(state["uinteger"])],
                  dtype=np.uint64)


def index_streams():
  out = {}
  for seed in range(8):
    for N in (10_000, 1_000_000):
      for n in (128, 1024):
        rng = np.random.default_rng(np.random.SeedSequence(seed).spawn(1)[0])
        before = pcg_words(rng.bit_generator.state)
        draws = np.stack([rng.choice(np.arange(0, N), size=n, replace=True)
                          for _ in range(3)]).astype(np.int32)
        after = pcg_words(rng.bit_generator.state)
        key = f"s{seed}_N{N}_n{n}"
        out[key + "_idx"] = draws
        out[key + "_before"] = before
        out[key + "_after"] = after
  np.savez_compressed(HERE / "index_streams.npz", **out)


def philox_kat():
  kat = [
      {"ctr": [0, 0, 0, 0], "key": [0, 0],
       "out": [0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8]},
      {"ctr": [0xFFFFFFFF] * 4, "key": [0xFFFFFFFF] * 2,
       "out": [0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD]},
      {"ctr": [0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344],
       "key": [0xA4093822, 0x299F31D0],
       "out": [0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1]},
  ]
  (HERE / "philox_kat.json").write_text(json.dumps(kat, indent=1))


def potential_kat():
  # tests/test_potential.py:66-92: lk = sum(sample * x), x rows = arange(4),
  # sample = ones(4); U = -sum(arange(4)) * obs - prior with prior = sum(sample)
  # = 4.  With a flat prior the expected value is -6 * obs.
  cases = []
  for obs in (7, 11):
    for dim in (3, 5):
      cases.append({"obs": obs, "dim": dim, "U_flat_prior": -6.0 * obs,
                    "U_sum_prior": -6.0 * obs - 4.0})
  (HERE / "potential_kat.json").write_text(json.dumps(cases, indent=1))


if __name__ == "__main__":
  index_streams()
  philox_kat()
  potential_kat()
  print("golden fixtures written to", HERE)
