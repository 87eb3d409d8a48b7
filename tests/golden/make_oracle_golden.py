"""Writes oracle_digests.json: digests of the CPU oracle's images on the small workloads.

    python tests/golden/make_oracle_golden.py

The cases are the seeded small scenes of the test suite (the 2,048-triangle plain draw at 256x256 and
reduced forms of the batched and blending workloads), so the file pins the oracle's behaviour: a later
change to kz_oracle.c that alters any pixel fails test_oracle_golden_digests."""
import hashlib
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
for p in (ROOT, os.path.dirname(HERE)):
    if p not in sys.path:
        sys.path.insert(0, p)


def cases():
    from kazan_gb300 import scenes
    import scene_cases
    out = {"small_soup": scenes.small_soup()}
    small = scene_cases.small_cases()
    for name in sorted(small):
        out["case_" + name] = small[name]
    return out


def main():
    from oracle import kz_oracle
    gold = {}
    for name, scene in cases().items():
        c, d, st = kz_oracle.render(scene, threads=4)
        gold[name] = {"color": hashlib.sha256(c.tobytes()).hexdigest()[:32],
                      "depth": hashlib.sha256(d.tobytes()).hexdigest()[:32], "fragments": st["fragments"]}
    with open(os.path.join(HERE, "oracle_digests.json"), "w", encoding="utf-8") as f:
        json.dump(gold, f, indent=1, sort_keys=True)
        f.write("\n")
    print(json.dumps(gold, indent=1))


if __name__ == "__main__":
    main()
