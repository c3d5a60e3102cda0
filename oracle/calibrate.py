"""Test infrastructure: how fast the oracle's FP32 port of
FluidSystemSPH::Run runs against the reference's own Run, both on one core
of this host, on the same seeded particles.  The benchmark's CPU baseline
times the port (the reference's sources do not travel to the GPU host), so
it reports this factor beside the baseline.  Needs the reference sources:

    python oracle/calibrate.py [/path/to/reference]

Writes oracle/port_calibration.json.
"""
from __future__ import annotations

import json
import os
import platform
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

import oracle as O  # noqa: E402


def main(ref_root: str, n: int = 8192, steps: int = 2) -> dict:
    O.build()
    if not O.build_ref(ref_root):
        raise SystemExit("reference harness did not build")
    rng = np.random.default_rng(3)
    # a block at spacing h/2 with jitter: the neighbourhoods of the workloads
    side = int(round(n ** (1 / 3)))
    g = np.stack(np.meshgrid(*[np.arange(side)] * 3, indexing="ij"), -1).reshape(-1, 3)[:n]
    pos = ((g - side / 2) * 0.02 + rng.uniform(-0.002, 0.002, g.shape)).astype(np.float32)
    prm = dict(g=(0.0, -9.81, 0.0), dt=1e-3, p0=1000.0, mass=0.008, visc=0.1, surf_tens=0.0728, k=3.0, cr=0.5,
               h=0.04, len=0.5)
    R = O.Reference()
    R.set_params(**prm)
    R.set_particles(pos)
    R.run(1)  # warm
    t0 = time.perf_counter()
    R.run(steps)
    t_ref = (time.perf_counter() - t0) / steps
    R.close()
    p = O.make_params(box_l=(0.5, 0.5, 0.5), **{k: v for k, v in prm.items() if k != "len"})
    O.run(p, pos, nsteps=1, nthreads=1)
    t0 = time.perf_counter()
    O.run(p, pos, nsteps=steps, nthreads=1)
    t_port = (time.perf_counter() - t0) / steps
    out = {"port_speed_over_reference": round(t_ref / t_port, 3),
           "reference_s_per_step": round(t_ref, 4), "port_s_per_step": round(t_port, 4),
           "note": (f"reference Run vs the oracle's FP32 port, {n} particles, 1 core, "
                    f"{platform.machine()} ({platform.processor() or 'cpu'}), gcc -O2 -ffp-contract=off; "
                    f"a value above 1 means the port is faster, so the CPU baseline flatters the reference")}
    with open(os.path.join(HERE, "port_calibration.json"), "w") as f:
        json.dump(out, f, indent=1)
        f.write("\n")
    return out


if __name__ == "__main__":
    print(json.dumps(main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")))
