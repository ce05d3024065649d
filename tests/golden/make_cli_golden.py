"""Generates tests/golden/cli_cases.json and tests/golden/cli_cases_ext.json:
for each case of tests/iwcli.py (case() and case_ext(), the latter with the
further options), the exit code of the reference's own imagew (built from its
sources by `make -C oracle refcli`) and the SHA-256 of the file it wrote.

    python tests/golden/make_cli_golden.py
"""
import json
import os
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))
import iwcli  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(HERE))
REF_CLI = os.path.join(ROOT, "oracle", "_ref", "imagew_ref")
N = 200
N_EXT = 300

if __name__ == "__main__":
    if not os.path.exists(REF_CLI):
        sys.exit("build the reference CLI first: make -C oracle refcli")
    for name, make, n in (("cli_cases.json", iwcli.case, N), ("cli_cases_ext.json", iwcli.case_ext, N_EXT)):
        out = []
        with tempfile.TemporaryDirectory() as d:
            for seed in range(n):
                c = make(seed)
                rc, digest = iwcli.run_case(REF_CLI, c, d)
                out.append({**c, "rc": rc, "sha256": digest})
        with open(os.path.join(HERE, name), "w") as f:
            json.dump(out, f, indent=0)
        print(name, len(out), "cases;", sum(1 for c in out if c["rc"] == 0), "written")
