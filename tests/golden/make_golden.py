"""Extract the reference's own known answers for the contour and k-mesh
generators, and the 2D lattice of the Kambe sums (unit-cell area, real and
reciprocal cell vectors as routine VECTOR2D prints them), from its sample run
sample/02-layer-scf (input_rsp.in, input_geo.in and the run log
Nb8_110.prn) into sample02_contour.json.

Run where a checkout of the reference tree exists, passing its root:
    python tests/golden/make_golden.py <path to the reference checkout>
The JSON it writes is committed; the tests only read the JSON.
"""
import json
import os
import re
import sys

if len(sys.argv) != 2:
    sys.exit("usage: make_golden.py <path to the reference checkout>")
ref = sys.argv[1]
d = os.path.join(ref, "sample", "02-layer-scf")
rsp = open(os.path.join(d, "input_rsp.in")).read().splitlines()
geo = open(os.path.join(d, "input_geo.in")).read().splitlines()
prn = open(os.path.join(d, "Nb8_110.prn")).read().splitlines()

out = {"source": "sample/02-layer-scf (input_rsp.in, input_geo.in, Nb8_110.prn)"}
for i, line in enumerate(rsp):
    if "IMESH,NPANEL" in line:
        out["imesh"], out["npanel"] = [int(v) for v in line.split()[:2]]
    if "NEPANEL,EBOTTOM,ETOP,EPS" in line:
        f = line.split()
        out["nepanel"] = int(f[0])
        out["ebottom"], out["etop"], out["eps"] = float(f[4]), float(f[5]), float(f[6])
    if re.search(r"\bNTAB\s*$", line):
        ntab = int(line.split()[0])
        tab = [rsp[i + 1 + t].split()[:2] for t in range(ntab)]
        out["ksettab"] = [[int(a), int(b)] for a, b in tab]
for line in geo:
    if "i2dlat,a2d" in line:
        f = line.split()
        out["i2dlat"], out["a2d"] = int(f[0]), float(f[1])
    if "beta,delta" in line:
        f = line.split()
        out["beta"], out["delta"] = float(f[0]), float(f[1])
    if line.strip().endswith("idgroup"):
        out["idgroup"] = line.split()[0]
pat = re.compile(r"ie=\s*(\d+)\s+e=\s*(\S+)\s+(\S+)\s+nk=\s*(\d+)")
pts = []
for line in prn:
    m = pat.search(line)
    if m:
        pts.append([int(m.group(1)), float(m.group(2)), float(m.group(3)), int(m.group(4))])
for i, line in enumerate(prn):
    if "unit cell area:" in line and "area2d" not in out:
        out["area2d"] = float(line.split()[-1])
    if "real lattice unit cell in 2D:" in line and "a_vectors" not in out:
        out["a_vectors"] = [[float(v) for v in prn[i + j].split()] for j in (2, 3)]
    if "reciprocal lattice unit cell in 2D:" in line and "b_vectors" not in out:
        out["b_vectors"] = [[float(v) for v in prn[i + j].split()] for j in (2, 3)]
n = out["nepanel"]
out["energies"] = [[p[1], p[2]] for p in pts[:n]]
out["nk"] = [p[3] for p in pts[:n]]
assert [p[0] for p in pts[:n]] == list(range(1, n + 1))
json.dump(out, open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "sample02_contour.json"), "w"), indent=1)
print(json.dumps(out)[:400])
