"""Generate the golden fixtures under tests/golden/ (run in a container that has the
reference checkout; the fixtures are committed so that nothing reads it at test time).

* ``philox_kat.json`` — the three Philox4x32-10 known-answer vectors that the
  reference's own test suite holds (``test/test_random.jl:4-14``), extracted from that
  file as text by a regular expression (the reference is Julia and cannot run here).
* ``rule_strings.json`` — the rule-string presets of ``src/rules.jl:249-265`` (names and
  B/S strings), extracted the same way, for the host-side rule parser tests.

Usage: python tests/golden/make_golden.py <path-to-reference-checkout>
"""
import json
import os
import re
import sys

HERE = os.path.dirname(os.path.abspath(__file__))


def philox_vectors(src: str):
    pat = re.compile(
        r"philox4x32\(\(([^)]*)\),\s*\(([^)]*)\)\)\s*==\s*\(([^)]*)\)", re.S)
    out = []
    for ctr, key, res in pat.findall(src):
        h = lambda s: [int(x.strip(), 16) for x in s.split(",") if x.strip()]
        out.append({"ctr": h(ctr), "key": h(key), "out": h(res)})
    return out


def presets(src: str, name: str):
    m = re.search(name + r"\s*=\s*Dict\{Symbol,String\}\((.*?)\)\n", src, re.S)
    return dict(re.findall(r":(\w+)\s*=>\s*\"([^\"]+)\"", m.group(1)))


def main(ref: str):
    with open(os.path.join(ref, "test", "test_random.jl")) as f:
        kats = philox_vectors(f.read())
    assert len(kats) == 3, kats
    with open(os.path.join(HERE, "philox_kat.json"), "w") as f:
        json.dump({"source": "test/test_random.jl:4-14", "vectors": kats}, f, indent=1)
    with open(os.path.join(ref, "src", "rules.jl")) as f:
        src = f.read()
    rs = {"source": "src/rules.jl:249-265",
          "life": presets(src, "const LIFE_PRESETS"),
          "generations": presets(src, "const GENERATIONS_PRESETS")}
    with open(os.path.join(HERE, "rule_strings.json"), "w") as f:
        json.dump(rs, f, indent=1, sort_keys=True)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py <path-to-reference-checkout>")
    main(sys.argv[1])
