"""Writes reference_line_counts.json: the line count of every reference Fortran source
that the code in this repository cites as `name.f90:N-M`.  Run in a checkout that has the
reference tree (path given as the first argument); the test that uses the counts needs
only the JSON.

Where a file name occurs in several reference directories, the pks2map sources come
first, then the vendored HEALPix / FITS modules, then the RandomField modules."""
import json
import os
import sys

PREFERENCE = ("src/pks2map_src", "src/modules/External", "src/modules/RandomField")


def main(ref):
    counts = {}
    for sub in reversed(PREFERENCE):
        d = os.path.join(ref, sub)
        for name in sorted(os.listdir(d)):
            if name.endswith((".f90", ".F90")):
                with open(os.path.join(d, name), "rb") as f:
                    counts[name] = {"path": sub + "/" + name, "lines": f.read().count(b"\n")}
    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "reference_line_counts.json")
    with open(out, "w") as f:
        json.dump(counts, f, indent=0, sort_keys=True)
    print("wrote", out, len(counts), "files")


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
