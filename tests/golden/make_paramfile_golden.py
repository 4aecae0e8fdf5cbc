"""Golden parser inputs from the reference's own example parameter files.

Reads paramfiles/example_*.txt and the additions_*.txt files of the
reference tree and stores, per file, the (key, value) token pairs its
read_parameterfile sees (src/read_param.c:378-412: the first two
whitespace-separated tokens of every line with at least two, lines starting
with '%' skipped) in tests/golden/ref_paramfiles.json.  tests/test_host.py
writes them back as parameter files and parses them.

Run from the repository root with MGP_REFERENCE_SRC set to the reference's
src/ directory:  MGP_REFERENCE_SRC=<reference>/src python tests/golden/make_paramfile_golden.py
"""
import glob
import json
import os

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))


def tokens(path):
    out = []
    for line in open(path, errors="replace"):
        t = line.split()
        if len(t) < 2 or t[0].startswith("%"):
            continue
        out.append([t[0], t[1]])
    return out


def main():
    src = os.environ.get("MGP_REFERENCE_SRC", "")
    pdir = os.path.join(os.path.dirname(src), "paramfiles") if src else ""
    if not os.path.isdir(pdir):
        raise SystemExit("set MGP_REFERENCE_SRC to the reference's src/ directory")
    files = sorted(glob.glob(os.path.join(pdir, "example_*.txt")) + glob.glob(os.path.join(pdir, "additions_*.txt")))
    data = {os.path.basename(f): tokens(f) for f in files}
    with open(os.path.join(ROOT, "tests", "golden", "ref_paramfiles.json"), "w") as f:
        json.dump(data, f, indent=0)
    print(len(data), "files")


if __name__ == "__main__":
    main()
