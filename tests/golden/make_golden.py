"""Writes the golden fixtures of tests/golden/ from the oracle.

connections_4x4.json: the reference's find_conn triple (all_conn, mel, use)
of Heisenberg (PBC, Marshall rotation), transverse-field Ising (PBC, h=3)
and J1-J2 (PBC, J2=0.5) for three fixed 4x4 configurations: the FP64 oracle's
output, which tests/test_oracle.py pins to the reference's exact energies.
Run from the repository root: python tests/golden/make_golden.py
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle import operators as ref_ops  # noqa: E402

CONFIGS = np.array([
    [[1, 1, 1, 1], [1, 1, 1, 1], [1, 1, 1, 1], [1, 1, 1, 1]],
    [[1, -1, 1, -1], [-1, 1, -1, 1], [1, -1, 1, -1], [-1, 1, -1, 1]],
    [[1, 1, -1, -1], [-1, 1, 1, -1], [1, -1, -1, 1], [-1, -1, 1, 1]],
], dtype=np.int8)

OPERATORS = {
    "heisenberg": lambda s: ref_ops.heisenberg_find_conn(s, pbc=True),
    "ising": lambda s: ref_ops.ising_find_conn(s, h=3.0, pbc=True),
    "j1j2": lambda s: ref_ops.j1j2_find_conn(s, j2=0.5, pbc=True),
}


def build():
    out = {"configs": CONFIGS.tolist()}
    for name, fc in OPERATORS.items():
        conn, mel, use = fc(CONFIGS.astype(np.float64))
        out[name] = {"conn": np.asarray(conn).astype(np.int8).tolist(),
                     "mel": np.asarray(mel, dtype=np.complex128).real.tolist(),
                     "mel_imag": np.asarray(mel, dtype=np.complex128).imag.tolist(),
                     "use": np.asarray(use, dtype=bool).tolist()}
    return out


if __name__ == "__main__":
    with open(os.path.join(HERE, "connections_4x4.json"), "w") as f:
        json.dump(build(), f, separators=(",", ":"))
