"""Regenerates the golden fixtures in tests/golden/ from the reference itself.

Runs in the development container only (it needs the reference sources):
builds the drivers of oracle/ref_golden/ against the reference's own code with
`make -C oracle ref`, runs them and writes their output here.

    python tests/golden/make_golden.py
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))


def main():
    ref = os.environ.get("REF", "/root/reference")
    if not os.path.isdir(ref):
        sys.exit(f"reference sources not found at {ref}")
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "ref", f"REF={ref}"], check=True)
    out = subprocess.run([os.path.join(ROOT, "oracle", "_ref", "mappers_golden")], check=True,
                         capture_output=True, text=True).stdout
    with open(os.path.join(HERE, "ref_mappers.txt"), "w") as f:
        f.write(out)
    print("wrote ref_mappers.txt:", len(out.splitlines()), "cases")


if __name__ == "__main__":
    main()
