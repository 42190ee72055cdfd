"""How much faster the oracle's C port runs than the reference itself.

TEST INFRASTRUCTURE ONLY.  The GPU machine has no reference tree, so the
bench's CPU baselines there time the port (psim_oracle.c), which is pinned
bit-exact to the reference but faster per thread (SoA arrays, a stable
counting sort).  This script times both on the same workload and threads in
a container that has the reference rebuilt from its sources (oracle/_ref):
the reference's 4000-particle AO case (L = 21, 7 cells a side, cutOff 1.1,
wellDepth 0.25, gamma 1, dt 1e-3) for `steps` steps of its hot loop
(force, push, nextSystem, cell rebuild; system.cpp:187-211 without the
analysis sweep), with the same injected noise, and checks that the two end
in the same state.  Prints one JSON line.

    python oracle/speed_factor.py [steps]
"""
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))

from oracle import port, ref  # noqa: E402
from proteinsim2015_gb300 import init  # noqa: E402


def main(steps=200):
    if not ref.available() and not ref.build():
        sys.exit("the reference is not built here (oracle/build_ref.sh needs its sources)")
    n, box, cs, scale, dt = 4000, 21, 3, 7, 0.001
    settings = {"kT": 1.0, "wellDepth": 0.25, "cutOff": 1.1, "gamma": 1.0, "timeStep": dt,
                "nParticles": n, "velFreq": 1000, "seed": 90210, "mass": 1.0}
    pos0 = init.rsa(n, box, 1.0, seed=90210).reshape(-1)
    vel0 = init.maxwell(n, 1.0, seed=90211).reshape(-1)
    rad = np.full(n, 0.5)
    noise = np.random.default_rng(3).standard_normal(steps * n * 6)
    out = {"workload": "AO N=4000 L=21 scale=7, %d steps, injected noise" % steps,
           "cpu": os.cpu_count()}
    for threads in sorted({os.cpu_count() or 1, 1}, reverse=True):
        p_ref, v_ref = pos0.copy(), vel0.copy()
        z = [np.zeros(3 * n) for _ in range(3)]
        t0 = time.perf_counter()
        ref.run("AO", settings, n, box, cs, scale, steps, noise, p_ref, z[0], v_ref, z[1], z[2],
                rad, np.ones(n), threads=threads)
        t_ref = time.perf_counter() - t0
        port.set_threads(threads)
        st = port.State(pos0, rad, vel=vel0)
        g = port.geom(n, box, cs, scale)
        t0 = time.perf_counter()
        err, *_ = port.run(g, port.make_force(port.AO, 1.1, kT=1.0, well_depth=0.25),
                           port.vgb_coeffs(1.0, dt, 1.0), dt, st, steps, noise, vel_freq=1000)
        t_port = time.perf_counter() - t0
        assert err == 0
        same = bool(np.max(np.abs(st.pos - p_ref)) <= 1e-9)
        out["threads_%d" % threads] = {
            "reference_particle_steps_per_s": n * steps / t_ref,
            "port_particle_steps_per_s": n * steps / t_port,
            "port_over_reference": t_ref / t_port, "same_final_state": same}
    print(json.dumps(out))


if __name__ == "__main__":
    main(int(sys.argv[1]) if len(sys.argv) > 1 else 200)
