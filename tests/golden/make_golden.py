"""Writes tests/golden/golden.json: the reference's known answers for the
matching path plus SHA-256 pins of the seeded fixtures they are computed on.

Known answers (constants and counts asserted by the reference's own tests):
  ratio_match_regression_hash   crates/core/src/matching.rs:1880-1901
  candidate_pairs_counts        crates/core/src/matching.rs:1402-1413
  candidate_pairs_power_of_two  crates/core/src/matching.rs:1415-1452
  pairs = 48P - 177             crates/core/tests/perf_structure.rs:29-47
The fixture pins let a run on another machine prove it regenerated the same
inputs (the generator's f64 ln/cos come from the platform libm).

Run: python tests/golden/make_golden.py
"""
import hashlib
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "..", "..", "oracle"))
import oracle as O  # noqa: E402


def sha(x) -> str:
    return hashlib.sha256(x.tobytes()).hexdigest()


def main():
    a, b = O.match_fixture(21, 2000, 700)
    m = O.ratio_match(a, b, 0.8, True, threads=4)
    n = O.ratio_match(a, b, 0.95, False, threads=4)
    assert (len(m), O.pairs_hash(m)) == (1145, 0x22CA99B86722152D)
    assert (len(n), O.pairs_hash(n)) == (1282, 0x7D0CD9993D0C89E5)
    a7, b7 = O.match_fixture(21, 7300, 3000)
    out = {
        "regression_hash": {
            "fixture": {"seed": 21, "na": 2000, "extra": 700, "nb": int(len(b)), "sha256_a": sha(a),
                        "sha256_b": sha(b)},
            "mutual_0.8": {"count": 1145, "hash": "0x22ca99b86722152d"},
            "loose_0.95": {"count": 1282, "hash": "0x7d0cd9993d0c89e5"},
            "source": "crates/core/src/matching.rs:1900-1901",
        },
        "timing_fixture": {"seed": 21, "na": 7300, "extra": 3000, "nb_truncated": 7300,
                           "sha256_a": sha(a7), "sha256_b7300": sha(b7[:7300]),
                           "source": "crates/core/src/matching.rs:1686-1708"},
        "candidate_pairs": {
            "rig10_t2_c1_p0": 51 + 84,
            "rig80_spec": 1563 + 2100,
            "rig80_pow2_unbounded": 1563 + 2100 + 3 * 64,
            "rig80_pow2_zero": 1563 + 2100 - 3 * 136,
            "pairs_48P_minus_177": {str(p): 48 * p - 177 for p in (20, 40, 80, 160)},
            "source": "crates/core/src/matching.rs:1402-1452, crates/core/tests/perf_structure.rs:29-47",
        },
    }
    with open(os.path.join(HERE, "golden.json"), "w") as f:
        json.dump(out, f, indent=1)
    print(json.dumps(out, indent=1))


if __name__ == "__main__":
    main()
