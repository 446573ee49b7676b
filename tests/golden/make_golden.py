"""Generate tests/golden/ref_pins.json from the reference kernel itself.

Builds oracle/_ref/libmcxref.so from the reference sources (src/mcx_core.cl
compiled as host C++ in place, see oracle/Makefile), runs every case of
tests/cases.py:pin_cases() and the photon replays of REPLAY_PINS (each
replaying the reference's own baseline records) one reference thread at a
time, and records
SHA-256 digests of the raw output bits (per-thread energies, merged fluence
field, detected-photon records, saved seeds) plus a few readable values.
tests/test_oracle_pins.py recomputes the same digests with the oracle.

Run here, where the reference sources are present:
    python tests/golden/make_golden.py [--reference /path/to/mcxcl]
"""
import argparse
import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, os.path.join(ROOT, "tests"))

import oracle  # noqa: E402
import cases  # noqa: E402


def digest(a):
    if a is None:
        return None
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def summarize(res):
    e = np.asarray(res["energy"], np.float32)
    field = np.asarray(res["field_raw"], np.float32)
    return {
        "energy_sha": digest(e.view(np.uint32)),
        "field_sha": digest(np.asfortranarray(field).ravel(order="F").view(np.uint32)),
        "detp_sha": digest(np.asarray(res["detp"], np.float32).view(np.uint32)),
        "seeds_sha": digest(res["seeds"]),
        "energy_tot": float(e[:, 1].astype(np.float64).sum()),
        "energy_esc": float(e[:, 0].astype(np.float64).sum()),
        "field_sum": float(field.astype(np.float64).sum()),
        "ndet": int(np.asarray(res["detp"]).shape[1]) if np.asarray(res["detp"]).ndim == 2 else 0,
    }


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=os.environ.get("MCX_REFERENCE"),
                    help="the reference checkout (default: $MCX_REFERENCE)")
    args = ap.parse_args()
    if not args.reference:
        sys.exit("name the reference checkout with --reference or MCX_REFERENCE")
    oracle.build(args.reference)
    if not oracle.ref_available():
        sys.exit("reference harness could not be built from " + args.reference)
    out = {}
    for name, cfg, nthread in cases.pin_cases():
        r = oracle.run_reference(cfg, nthread=nthread, core=nthread)
        out[name] = dict(summarize(r), nthread=nthread)
        if name in cases.DETECT_AFTER_REFLECT:
            # the records themselves (float bits), for the subset check
            out[name]["detp_bits"] = np.asarray(r["detp"], np.float32).T.view(np.uint32).tolist()
        print(name, out[name]["ndet"], out[name]["energy_tot"])
    # polarised transport: Mueller rows and properties from the reference's own Mie
    # routine, stored with the pin (the oracle takes them as inputs)
    pcfg = cases.pol_inputs(cases.polarized(), oracle.ref_mie)
    r = oracle.run_reference(pcfg, nthread=128, core=128)
    out["polarized"] = dict(summarize(r), nthread=128, smatrix=pcfg["smatrix"].ravel().tolist(),
                            prop=np.asarray(pcfg["prop"], np.float32).ravel().tolist())
    print("polarized", out["polarized"]["ndet"], out["polarized"]["energy_tot"])
    for name, bkw, rkw, nthread in cases.REPLAY_PINS:
        base = cases.small_two_media(**bkw)
        b = oracle.run_reference(base, nthread=128, core=128)
        cfg = cases.replay_cfg(base, b["detp"], b["seeds"], **rkw)
        r = oracle.run_reference(cfg, nthread=nthread, core=nthread, nblocksize=16)
        out[name] = dict(summarize(r), nthread=nthread)
        print(name, out[name]["ndet"], out[name]["field_sum"])
    for name, kw in cases.TRAJ_PINS:
        r = oracle.run_reference(cases.small_two_media(**kw), nthread=128, core=128)
        out[name] = dict(summarize(r), nthread=128, ntraj=r["ntraj"], traj_sha=cases.traj_digest(r["traj"]))
        print(name, r["ntraj"])
    with open(os.path.join(HERE, "ref_pins.json"), "w") as f:
        json.dump(out, f, indent=1, sort_keys=True)


if __name__ == "__main__":
    main()
