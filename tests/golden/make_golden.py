"""Extract the reference's lid-driven-cavity fixtures into tests/golden/.

Sources, both in TEST/DrivenCavity/ of the reference tree:
- prof_j.0000.dat: u, v, rho at x = 128 of the 256^2 Re=100 cavity, one block per 2500 steps.
  The t = 0, 2500 and 20000 blocks are kept (ldc256_prof_j_ref.txt).
- ghia.y.dat: the centre-line u(y)/U table the reference's plot.R*.gnu scripts compare
  against, copied unchanged (ghia_y_ref.txt).
Run where the reference tree is mounted:  python tests/golden/make_golden.py /path/to/reference
"""
import os
import sys

ref = os.path.join(sys.argv[1] if len(sys.argv) > 1 else "/root/reference", "TEST", "DrivenCavity")
here = os.path.dirname(os.path.abspath(__file__))
src = os.path.join(ref, "prof_j.0000.dat")
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
dst = os.path.join(here, "ldc256_prof_j_ref.txt")
with open(dst, "w") as f:
    f.write("".join(out))
print(dst, len(out), "lines")
ghia = open(os.path.join(ref, "ghia.y.dat")).read()
dst = os.path.join(here, "ghia_y_ref.txt")
with open(dst, "w") as f:
    f.write(ghia)
print(dst, ghia.count("\n"), "lines")
