"""Regenerate the golden fixtures of tests/golden/ from the CPU oracle.

The reference ships no golden outputs (and cannot be run on Linux), so these
fixtures freeze the oracle's FP32 and FP64 results of a few small seeded cases:
they pin the oracle against regressions and give the GPU tests a committed
target.  Run from the repository root:  python tests/golden/make_golden.py
"""
import json
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from oracle.binding import Oracle  # noqa: E402
from zq_smokesimulation_gb300 import capi  # noqa: E402
from zq_smokesimulation_gb300 import workloads as wl  # noqa: E402

CASES = [
    # name, dims, seed, K, substeps, closed, vel_mode, sca_mode, steps
    ("open_mac_9x8x7", (9, 8, 7), 7, 12, 4, False, capi.ADV_VEL_INMAC_OUTMAC, capi.ADV_SCA_MAC, 2),
    ("closed_reg_8x9x6", (8, 9, 6), 21, 10, 3, True, capi.ADV_VEL_INREG_OUTREG, capi.ADV_SCA_REG, 2),
    ("open_regmac_6x5x7", (6, 5, 7), 5, 8, 2, False, capi.ADV_VEL_INREG_OUTMAC, capi.ADV_SCA_MAC, 3),
]


def main():
    out = Path(__file__).resolve().parent
    o32, o64 = Oracle(np.float32), Oracle(np.float64)
    for name, dims, seed, K, sub, closed, vm, sm, steps in CASES:
        w = wl.small_case(*dims, seed=seed, K=K, substeps=sub, closed=closed, vel_mode=vm, sca_mode=sm)
        arrays = {}
        for o, tag in ((o32, "f32"), (o64, "f64")):
            st = o.state(w)
            rc, _ = o.step(w.W, w.H, w.D, st, w.occ, w.params, steps)
            assert rc == 0
            for k in ("u", "v", "w", "T", "rho"):
                arrays[f"{tag}_{k}"] = st[k]
        meta = {"dims": list(dims), "seed": seed, "K": K, "substeps": sub, "closed": closed, "vel_mode": vm,
                "sca_mode": sm, "steps": steps}
        np.savez_compressed(out / f"{name}.npz", meta=json.dumps(meta), **arrays)
        print("wrote", name)


if __name__ == "__main__":
    main()
