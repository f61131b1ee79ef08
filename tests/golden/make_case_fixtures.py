"""Generate tests/golden/cases.json and tests/golden/case_masks.npz from the
reference's sample cases (samples/**/*.dat and the .bmp beside each 2-D
case), read by the case-file oracle (oracle/case_oracle.py).

Run from the repository root where the reference tree exists:
    python tests/golden/make_case_fixtures.py [reference root]
(default: LATTIBOL_REF_DIR, else the oracle recipe's default location)

cases.json holds, per case, the parsed parameters (floats as IEEE-754 bit
patterns) and, for 2-D cases, the mask's size, solid count and SHA-256; for
3-D cases the voxelisation of the STL surface at the case's max_dim (size,
solid count, SHA-256).  case_masks.npz holds each distinct 2-D mask
bit-packed, case_stl.npz each distinct STL surface as float32 triangles.  The tests need neither
the reference nor this script.
"""
import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import case_oracle  # noqa: E402


def fbits(v):
    return "%08x" % int(np.float32(v).view(np.uint32))


def params_json(p):
    out = {}
    for k, v in p.items():
        if isinstance(v, list):
            out[k] = [fbits(x) for x in v]
        elif isinstance(v, (int, np.integer)) and not isinstance(v, np.floating):
            out[k] = int(v)
        else:
            out[k] = fbits(v)
    return out


def main(ref_root):
    samples = os.path.join(ref_root, "samples")
    cases, masks, triangles = [], {}, {}
    for dirpath, _dirs, files in sorted(os.walk(samples)):
        for fn in sorted(files):
            if not fn.endswith(".dat"):
                continue
            dat = os.path.join(dirpath, fn)
            rel = os.path.relpath(dat, samples)
            p = case_oracle.load_parameters(dat)
            entry = {"name": rel, "params": params_json(p)}
            bmp = dat[:-3] + "bmp"
            stl = dat[:-3] + "stl"
            if p["max_dim"] > 1 and os.path.exists(stl):
                tri = case_oracle.read_stl(stl)
                key = "t_" + hashlib.sha256(tri.tobytes()).hexdigest()[:16]
                triangles[key] = tri
                mask = case_oracle.voxelize(tri, p["max_dim"])
                entry.update(stl=key, stl_dims=list(mask.shape[::-1]),
                             stl_solids=int(mask.sum()),
                             stl_sha256=hashlib.sha256(mask.tobytes()).hexdigest())
            if p["max_dim"] <= 1 and os.path.exists(bmp):
                w, h, mask = case_oracle.load_solids_bmp(bmp)
                sha = hashlib.sha256(mask.tobytes()).hexdigest()
                entry.update(width=w, height=h, solids=int(mask.sum()), mask=sha[:16],
                             sha256=sha)
                masks["m_" + sha[:16]] = np.packbits(mask.reshape(-1))
            cases.append(entry)
    with open(os.path.join(HERE, "cases.json"), "w") as fh:
        json.dump(cases, fh, indent=1)
    np.savez_compressed(os.path.join(HERE, "case_masks.npz"), **masks)
    np.savez_compressed(os.path.join(HERE, "case_stl.npz"), **triangles)
    print("%d cases, %d distinct masks, %d distinct STL surfaces"
          % (len(cases), len(masks), len(triangles)))


if __name__ == "__main__":
    import lb_oracle
    main(sys.argv[1] if len(sys.argv) > 1 else lb_oracle.ref_dir())
