"""Pins of the host-side formats against the reference's own code.

Runs the reference's configuration layer and writers, compiled in place from
the reference checkout by `make -C oracle ref` (oracle/ref_utils.c), and
stores what they produce in tests/golden/ref_host_pins.json:

* "json": for each built-in benchmark input (tests/golden/bench_*.json), the
  configuration the reference's mcx_readconfig loads -- the scalars, the
  volume size, and SHA-256 digests of the volume words (labels and
  detector-mask bits after preprocessing), the media rows and the detector
  rows -- so the library's JSON reader can be checked without the reference.
* "writers": seeded synthetic detected-photon records with their seeds, the
  SHA-256 of the .mch file the reference's mcx_savedetphoton writes for
  them, and the reference's .jdat (mcx_savejdet) and .jnii (mcx_savejnii)
  documents themselves.
* "adjoint": seeded fields and the SHA-256 of what the reference's adjoint
  post-kernels (mcx_adjoint_kernel, mcx_adjoint_dcoeff_kernel,
  src/mcx_core.cl:3393-3512, compiled on the host) compute from them.

    python tests/golden/make_host_pins.py --reference <reference checkout>
"""
import argparse
import base64
import glob
import hashlib
import json
import os
import sys
import tempfile
import zlib

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import oracle  # noqa: E402


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def writer_inputs():
    """Synthetic records: 9 photons, 2 media, savedetflag dspmxvw (0x7F):
    detid, nscat x2, ppath x2, mom x2, p x3, v x3, w0 -> 14 columns."""
    rng = np.random.default_rng(20251204)
    n, m = 9, 2
    cols = [rng.integers(1, 5, (n, 1)).astype(np.float32),             # detector id
            rng.integers(0, 60, (n, m)).astype(np.float32),            # scatter counts (by value)
            (rng.random((n, m)) * 20).astype(np.float32),              # partial paths
            rng.random((n, m)).astype(np.float32),                     # momentum transfer
            (rng.random((n, 3)) * 60).astype(np.float32),              # exit position
            rng.standard_normal((n, 3)).astype(np.float32),            # exit direction
            rng.random((n, 1)).astype(np.float32)]                     # initial weight
    detp = np.concatenate(cols, axis=1)
    seeds = rng.integers(0, 256, (n, 16)).astype(np.uint8)
    hist = [1, m, 4, detp.shape[1], 1000000, n + 5, n, 16, 1, 1, 0x7F, 1]
    histf = [1.0, 0.0123456789]
    prop = [[0, 0, 1, 1], [0.005, 1.0, 0.01, 1.37], [0.002, 5.0, 0.9, 1.0]]
    vol = np.random.default_rng(7).random((6, 5, 4, 3)).astype(np.float32)
    return dict(detp=detp, seeds=seeds, hist=hist, histf=histf, prop=prop, vol=vol)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=os.environ.get("MCX_REFERENCE"),
                    help="the reference checkout (default: $MCX_REFERENCE)")
    args = ap.parse_args()
    if not args.reference:
        sys.exit("name the reference checkout with --reference or MCX_REFERENCE")
    oracle.build(args.reference)
    if not oracle.refutils_available():
        sys.exit("the reference's host layer could not be built from " + args.reference)
    out = {"json": {}, "writers": {}}
    for path in sorted(glob.glob(os.path.join(HERE, "bench_*.json"))):
        name = os.path.basename(path)[6:-5]
        r = oracle.ref_readconfig(path)
        out["json"][name] = {
            "scalars": {k: (float(r[k]) if isinstance(r[k], float) else int(r[k])) for k in oracle.CONFIG_SCALARS},
            "dim": [int(x) for x in r["dim"]],
            "srcpos": r["srcpos"].tolist(), "srcdir": [float(x) for x in r["srcdir"]],
            "srcparam1": r["srcparam1"].tolist(), "srcparam2": r["srcparam2"].tolist(),
            "vol_sha": sha(r["vol"]), "prop_sha": sha(r["prop"]), "detpos_sha": sha(r["detpos"]),
            "labels": np.unique(r["vol"] & 0x7FFFFFFF).tolist(), "masked": int((r["vol"] >> 31).sum()),
        }
        print(name, r["dim"], out["json"][name]["labels"], out["json"][name]["masked"])
    w = writer_inputs()
    with tempfile.TemporaryDirectory() as tmp:
        cwd = os.getcwd()
        os.chdir(tmp)
        try:
            oracle.ref_savedet("ref", w["hist"], w["histf"], w["prop"], w["detp"], w["seeds"], 1, 0)
            oracle.ref_savedet("ref", w["hist"], w["histf"], w["prop"], w["detp"], w["seeds"], 1, 1)
            oracle.ref_savejnii(w["vol"], (0.5, 0.5, 0.5), "vol", session="pins", maxgate=3, outputtype=1)
            mch = open("ref.mch", "rb").read()
            jdat = json.load(open("ref_detp.jdat"))
            jnii = json.load(open("vol.jnii"))
        finally:
            os.chdir(cwd)
    out["writers"] = {"detp": w["detp"].tolist(), "seeds": w["seeds"].tolist(), "hist": w["hist"],
                      "histf": w["histf"], "prop": w["prop"], "vol": w["vol"].ravel(order="F").tolist(),
                      "vol_shape": list(w["vol"].shape), "mch_sha": hashlib.sha256(mch).hexdigest(),
                      "mch_size": len(mch), "jdat": jdat, "jnii": jnii}
    # the adjoint post-kernels on a seeded field: 9 x 8 x 7 voxels, 2 gates,
    # one source and two detectors (and a 2-voxel-wide edge case in x)
    out["adjoint"] = []
    for shape in ((9, 8, 7), (2, 5, 4)):
        nx, ny, nz = shape
        ns, nd, maxgate = 1, 2, 2
        field = np.random.default_rng(99).random((nx, ny, nz, maxgate, ns + nd)).astype(np.float32)
        case = {"shape": list(shape), "ns": ns, "nd": nd, "maxgate": maxgate,
                "field_zlib_b64": base64.b64encode(zlib.compress(field.ravel(order="F").tobytes())).decode()}
        for kind in (0, 1):
            case["sha%d" % kind] = sha(oracle.ref_adjoint(kind, field, ns, nd, nx, ny, nz, maxgate))
        out["adjoint"].append(case)
    with open(os.path.join(HERE, "ref_host_pins.json"), "w") as f:
        json.dump(out, f, indent=1, sort_keys=True)
        f.write("\n")
    print("mch", len(mch), "bytes")


if __name__ == "__main__":
    main()
