"""Generate the committed golden fixtures (small .npz files) from the FP64 oracle.

Run from the repository root:  python tests/golden/make_fixtures.py [name ...]
(no names: every fixture; names: only those, e.g. `sf`, leaving the others' files untouched)
Each fixture stores the FP32 input the GPU receives and the FP64 oracle output for a
geometry defined in tests/cases.py.  The oracle itself is pinned by tests/test_oracle.py
against the reference's known answers and conservation tests
(tests/golden/reference_known_answers.json).
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, os.path.join(ROOT, "tests"))
import cases as C  # noqa: E402
import oracle as O  # noqa: E402


def main():
    out = {}
    c = C.FDK_FLAT
    proj = O.ellipsoid_proj(c["rg"], C.ELL3).astype(np.float32)
    out["fdk_flat"] = dict(proj=proj, ref=O.fdk(c["rg"], c["ig"], proj, shape=c["window"]))
    c = C.FDK_ARC_SHORT
    mask = C.cyl_mask(c["ig"], c["mask_r"])
    proj = O.ellipsoid_proj(c["rg"], C.ELL3).astype(np.float32)
    out["fdk_arc_short"] = dict(proj=proj, ref=O.fdk(c["rg"], dict(c["ig"], mask=mask), proj, shape=c["window"],
                                                     cutoff=c["cutoff"]))
    for name, c in (("fbp_par", C.PAR), ("fbp_arc_short", C.ARC_SHORT), ("fbp_flat", C.FLAT)):
        s = O.ellipse_sino(c["rg"], C.ELL2).astype(np.float32)
        out[name] = dict(sino=s, ref=O.fbp(c["rg"], c["ig"], s, shape=c["window"]))
    rng = np.random.default_rng(7)
    f = C.FILTER_WRAP
    x = rng.standard_normal((f["rows"], f["nb"])).astype(np.float32)
    Hk = O.fbp_filter(dict(kind="flat", nb=f["nb"], d=1.0), npad=f["npad"])
    out["sino_filter_wrap"] = dict(x=x, Hk=Hk, ref=O.sino_filter(x, Hk, extra=f["extra"]))
    g = C.BDD
    geo = O.bdd_geo(g["DSD"], g["DS0"], g["pSize"], g["dSize"], g["nPix"], g["nDet"], g["angle"])
    ph = rng.random((g["nPix"], g["nPix"])).astype(np.float32)
    y = rng.random((g["nDet"], len(g["angle"]))).astype(np.float32)
    out["bdd"] = dict(phantom=ph, sino=y, ref_proj=O.project_bdd(ph, geo), ref_back=O.backproject_bdd(y, geo))
    sf = {}
    rs = np.random.default_rng(11)
    for kind, c in C.SF.items():
        nx, ny = c["ig"]["dims"]
        img = rs.random((ny, nx)).astype(np.float32)
        sn = rs.random((c["rg"]["na"], c["rg"]["nb"])).astype(np.float32)
        sf.update({f"{kind}_image": img, f"{kind}_sino": sn, f"{kind}_ref_proj": O.sf_project(c["rg"], c["ig"], img),
                   f"{kind}_ref_back": O.sf_back(c["rg"], c["ig"], sn)})
    out["sf"] = sf
    wanted = set(sys.argv[1:])
    for name, d in out.items():
        if wanted and name not in wanted:
            continue
        np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **d)
        print("wrote", name)


if __name__ == "__main__":
    main()
