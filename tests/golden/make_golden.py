"""Extract the reference's golden values for the hot path into he1d_golden.json.

Usage: python make_golden.py <path to the CodyFortran sources>, or with the
path in $CODY_REFERENCE; there is no default.  The values are read from the reference's own
test programs (their `check(error, value, golden, thr=...)` calls), so the
JSON is a verbatim record of what the reference tests assert.
"""
import json
import os
import re
import sys


def reference_root():
    """The CodyFortran checkout: first argument, else $CODY_REFERENCE."""
    if len(sys.argv) > 1:
        return sys.argv[1]
    if os.environ.get("CODY_REFERENCE"):
        return os.environ["CODY_REFERENCE"]
    sys.exit("make_golden.py: give the CodyFortran source directory as the argument or in $CODY_REFERENCE")


TESTS = {
    "he1d_01_exact_diag": "test/simulationTests/He1d/T_He1d_01_ExactDiagGridBasedFullExpansion.f90",
    "he1d_02_tdci_exact_diag": "test/simulationTests/He1d/T_He1d_02_ExactDiagTdci.f90",
    "he1d_03_tdhf_imag": "test/simulationTests/He1d/T_He1d_03_ImagTimePropagationTdhx.f90",
    "he1d_04_mctdhf_imag": "test/simulationTests/He1d/T_He1d_04_ImagTimePropagationMctdhx.f90",
    "he1d_05_mctdhf_split_rk4": "test/simulationTests/He1d/T_He1d_05_TimePropagationMctdhx.f90",
    "he1d_06_mctdhf_split_sil": "test/simulationTests/He1d/T_He1d_06_TimePropagationMctdhxSil.f90",
    "he1d_07_mctdhf_imag_restricted": "test/simulationTests/He1d/T_He1d_07_ImagTimePropagationMctdhxRestricted.f90",
    "fedvr_derivative": "test/componentTests/Utils/T_Utils_DerivativeFedvr.f90",
}
PAT = re.compile(r"call check\(error,\s*([^,]+),\s*([-+0-9.eE_R64]+)?,?\s*(?:thr=([-+0-9.eE_R64]+))?")


def main():
    REF = reference_root()
    out = {}
    for key, rel in TESTS.items():
        path = os.path.join(REF, rel)
        checks = []
        with open(path) as f:
            for lineno, line in enumerate(f, 1):
                if "call check(" not in line:
                    continue
                m = re.search(r"call check\(error,\s*(.*)\)\s*$", line.strip())
                args = [a.strip() for a in m.group(1).split(",")] if m else []
                entry = {"line": lineno, "args": args}
                for a in args:
                    v = a.split("=")[-1].replace("_R64", "")
                    try:
                        float(v)
                    except ValueError:
                        continue
                    if a.startswith("thr="):
                        entry["thr"] = float(v)
                    elif "golden" not in entry:
                        entry["golden"] = float(v)
                checks.append(entry)
        out[key] = {"file": rel, "checks": checks}
    json.dump(out, open(os.path.join(os.path.dirname(__file__), "he1d_golden.json"), "w"), indent=1)


if __name__ == "__main__":
    sys.exit(main())
