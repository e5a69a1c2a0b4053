"""Writes tests/golden/long_horizon_hashes.json: sha256 hashes of all six
fields (ghost cells included) of the oracle's state at checkpoints of the two
plain workloads, for bit-exact comparison of long GPU runs.

* N = 64 (size 66): tests.util.small_workload, 100 frames, checkpoints 1, 10, 100.
* N = 1024 (size 1026): bench.scene(seed 2) with the sources of a 1000-frame
  draw, 1000 frames, checkpoints 1, 10, 100, 1000.

The oracle is the C++ restatement of fluid.rs (oracle/); the 1000-frame run
takes tens of minutes on one host core. Run from the repository root:
    python tests/golden/make_long_hashes.py
"""
import json
import os
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import bench  # noqa: E402
import oracle  # noqa: E402
from tests.util import small_workload, state_hashes  # noqa: E402

OUT = os.path.join(HERE, "long_horizon_hashes.json")


def run(name, size, iters, dt, dv, rects, sx, sy, sd, su, sv, checkpoints):
    f = oracle.OracleFluid(size, dt, iters, dv, dv)
    for r in rects:
        f.fill_obstacle(*r)
    out, done, t0 = {}, 0, time.time()
    for upto in checkpoints:
        f.run(upto - done, sx[done:upto], sy[done:upto], sd[done:upto], su[done:upto],
              sv[done:upto])
        done = upto
        out[str(upto)] = state_hashes(f.fields)
        print(f"{name}: frame {upto} ({time.time() - t0:.0f} s)", flush=True)
    return out


def main():
    oracle.build()
    res = {"fields": list(oracle.FIELDS), "hash": "sha256 of each field's float32 bytes"}
    size, iters, dt, dv, rect, xs, ys, d, u, v = small_workload(100)
    res["n64"] = {"size": size, "iters": iters, "delta_t": dt, "diffusion": dv,
                  "viscosity": dv, "rects": [list(rect)], "frames": 100,
                  "workload": "tests.util.small_workload(100)",
                  "checkpoints": run("n64", size, iters, dt, dv, [rect], xs, ys, d, u, v,
                                     (1, 10, 100))}
    nfr = 1000
    rects, sx, sy, sd, su, sv = bench.scene(bench.SEED, nfr)
    res["n1024"] = {"size": bench.SIZE, "iters": bench.ITERS, "delta_t": bench.DT,
                    "diffusion": bench.DIFF, "viscosity": bench.VISC,
                    "rects": [list(r) for r in rects], "frames": nfr,
                    "workload": f"bench.scene({bench.SEED}, {nfr})",
                    "checkpoints": run("n1024", bench.SIZE, bench.ITERS, bench.DT, bench.DIFF,
                                       rects, sx, sy, sd, su, sv, (1, 10, 100, 1000))}
    with open(OUT, "w") as fh:
        json.dump(res, fh, indent=1)
    print("wrote", OUT)


if __name__ == "__main__":
    main()
