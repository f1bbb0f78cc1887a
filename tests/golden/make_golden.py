"""Generate the golden fixtures that pin the oracle (run from the repo root):

    python tests/golden/make_golden.py

* ``ed_energies.json``: exact ground energies (scipy sparse Lanczos in the S^z = 0
  sector) of open Heisenberg chains and of a small J1-J2 cylinder.  The reference ships no
  golden vectors for the sweep path (its tests assert nothing), so exact diagonalisation
  is the independent anchor.
* ``quench_sz.json``: exact <S^z_i(t)> of the open Heisenberg chain (N = 12) after a quench
  from the Neel state (site 0 Up), real-time evolution by expm_multiply at t = 0.5 and 1.0:
  the small-N analogue of the real-time TDVP workload (N = 64, dt = 0.05).
"""
from __future__ import annotations

import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import ed  # noqa: E402
from oracle import tn_oracle as O  # noqa: E402


def main():
    out = {"heisenberg_chain": {}, "j1j2_cylinder": {}}
    for N in (6, 8, 10, 12, 14, 16, 20):
        out["heisenberg_chain"][str(N)] = ed.ground_energy(N, ed.heisenberg_chain_terms(N))
    for (Lx, Ly) in ((3, 4), (4, 4)):
        terms = O.j1j2_cylinder_terms(Lx, Ly, 1.0, 0.5)
        out["j1j2_cylinder"][f"{Lx}x{Ly}"] = ed.ground_energy(Lx * Ly, terms)
    with open(os.path.join(HERE, "ed_energies.json"), "w") as f:
        json.dump(out, f, indent=1, sort_keys=True)
    print(json.dumps(out, indent=1))
    N, times = 12, [0.5, 1.0]
    q = {"N": N, "times": times, "up_sites": list(range(0, N, 2)),
         "sz": ed.quench_sz(N, ed.heisenberg_chain_terms(N), range(0, N, 2), times)}
    with open(os.path.join(HERE, "quench_sz.json"), "w") as f:
        json.dump(q, f, indent=1)
    print(json.dumps(q))


if __name__ == "__main__":
    main()
