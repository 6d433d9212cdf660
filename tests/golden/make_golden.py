"""Extract the reference's lid-driven-cavity profile fixture into tests/golden/.

Source: TEST/DrivenCavity/prof_j.0000.dat of the reference tree (u, v, rho at x = 128 of the
256^2 Re=100 cavity, one block per 2500 steps).  The t = 0, 2500 and 20000 blocks are kept.
Run where the reference tree is mounted, naming its root as the argument or in
BGK2D_REFERENCE_ROOT:  python tests/golden/make_golden.py /path/to/reference
"""
import os
import sys

root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("BGK2D_REFERENCE_ROOT", "")
if not root:
    sys.exit("usage: make_golden.py <reference root>  (or set BGK2D_REFERENCE_ROOT)")
src = os.path.join(root, "TEST", "DrivenCavity", "prof_j.0000.dat")
keep = {0, 2500, 20000}
out = []
cur = None
for line in open(src):
    if line.startswith("#"):
        cur = int(line.split("=")[1])
        if cur in keep and f"# t={cur}\n" not in out:
            out.append(f"# t={cur}\n")
        else:
            cur = None
        continue
    if cur is not None and line.strip():
        out.append(line)
dst = os.path.join(os.path.dirname(os.path.abspath(__file__)), "ldc256_prof_j_ref.txt")
with open(dst, "w") as f:
    f.write("".join(out))
print(dst, len(out), "lines")
