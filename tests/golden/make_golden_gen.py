"""Generate the generalized-grid and 2D-scheme golden vectors in
tests/golden/gen/ from the reference itself.

The reference's gen2d.cpp / gen3d.cpp / cart2d.cpp (with metric.hpp, flux.hpp,
presgrad.hpp, velocity.hpp), compiled unmodified by oracle/ref_build.sh, run
small seeded cases.  Per case it stores:
  X   node coordinates (ni, nj, nk, 3) — a smoothly distorted box
  MT  the metric tensor after preSim (zeros on cartesian cases)
  U0  initial state with ghosts filled (applyBCs of the seeded interior;
      the generalized modules never fill ghosts themselves)
  R1  one compute() of U0
  UN  the state after `steps` time steps
Needs the reference tree (FST_REFERENCE or /root/reference).

    python tests/golden/make_golden_gen.py
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.abspath(os.path.join(HERE, "..", ".."))
sys.path.insert(0, ROOT)

from fiesta_gb300 import abi  # noqa: E402
from fiesta_gb300.solver import initial_conditions  # noqa: E402
from oracle.oracle import Reference, build_reference  # noqa: E402
from tests.golden_io import wavy_nodes  # noqa: E402

SP3 = [dict(gamma=1.4, M=1.0, mu=1.8e-5), dict(gamma=1.67, M=0.5, mu=2e-5),
       dict(gamma=1.3, M=2.0, mu=1.5e-5)]
GEN = abi.GRID_GENERALIZED


def cases():
    unit = (1.0, 1.0, 1.0)  # generalized decks set dx = dy = dz = 1 (src/input.cpp:344-350)
    return [
        ("gen2d_weno", abi.make_config(2, (20, 16), dx=unit, dt=2e-4, species=SP3[:2], R=1.0,
                                       grid_type=GEN), 0.25, 12),
        ("gen2d_quick", abi.make_config(2, (17, 14), dx=unit, dt=2e-4, species=SP3[:1], R=1.0,
                                        grid_type=GEN, scheme="quick", ceq=True), 0.2, 10),
        ("gen2d_centered", abi.make_config(2, (15, 18), dx=unit, dt=1e-4, species=SP3[:2], R=1.0,
                                           grid_type=GEN, scheme="centered4"), 0.2, 10),
        ("cart2d_quick", abi.make_config(2, (19, 13), dt=2e-4, species=SP3[:2], R=1.0, visc=True,
                                         ceq=True, scheme="quick",
                                         bcs=("outflow", "reflective", "noslip", "hydrostatic",
                                              "outflow", "outflow")), 0.0, 10),
        ("cart2d_centered", abi.make_config(2, (14, 17), dt=1e-4, species=SP3[:3], R=1.0,
                                            scheme="centered4", buoyancy=True, g=0.5,
                                            rho_ref=1.0, periodic=(True, False, False)), 0.0, 10),
        ("gen3d_weno", abi.make_config(3, (9, 8, 7), dx=unit, dt=1e-4, species=SP3, R=1.0,
                                       grid_type=GEN, visc=True, ceq=True), 0.25, 6),
    ]


def main():
    if not Reference.available():
        build_reference()
    os.makedirs(os.path.join(HERE, "gen"), exist_ok=True)
    for name, cfg, amp, steps in cases():
        gen = cfg.grid_type == GEN
        U0 = initial_conditions(cfg, abi.IC_RANDOM_SMOOTH, seed=len(name) * 7 + steps)
        X = wavy_nodes(cfg, amp=amp)
        r = Reference(cfg)
        r.set_state(U0)
        r.apply_bcs()  # finite ghosts for the generalized cases
        U0 = r.get_state()
        if gen:
            r.set_grid(X)
            MT = r.metrics()
        else:
            MT = np.zeros((1,))
        R1 = r.compute_rhs()
        r = Reference(cfg)
        r.set_state(U0)
        if gen:
            r.set_grid(X)
        r.rk_step(steps)
        UN = r.get_state()
        meta = dict(name=name, config=abi.config_to_dict(cfg), steps=steps, amp=amp,
                    source="reference sources compiled by oracle/ref_build.sh")
        path = os.path.join(HERE, "gen", f"{name}.npz")
        np.savez_compressed(path, X=X, MT=MT, U0=U0, R1=R1, UN=UN, meta=json.dumps(meta))
        assert np.isfinite(UN).all() and np.isfinite(R1).all(), name
        print(f"{name}: {os.path.getsize(path) / 1024:.0f} KiB, |R1|max={np.abs(R1).max():.3g}")


if __name__ == "__main__":
    main()
