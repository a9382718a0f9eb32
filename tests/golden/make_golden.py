"""Generate the golden vectors in tests/golden/ from the reference itself.

Runs the reference's own FP64 sources (cart2d.cpp, cart3d.cpp, bc.cpp, rk.cpp
and the kernel headers, compiled unmodified against a host Kokkos shim by
oracle/ref_build.sh) on small seeded cases and stores, per case:
  U0  initial state (LayoutLeft, ghosts included)
  R1  applyBCs on U0, then one cart{2,3}d_func::compute() (3D applies BCs
      again inside compute, which is idempotent)
  UN  state after `steps` time steps (preStep, rkAdvance, postStep)
  SN  secondary variables (copyExtraVars) of UN
and the run config as JSON.  Needs the reference tree (FST_REFERENCE or
/root/reference); the fixtures it writes are what travels.

    python tests/golden/make_golden.py
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

AIR = dict(gamma=1.4, M=0.02896, mu=1.8e-5)
HE = dict(gamma=1.67, M=0.004, mu=1.99e-5)
SP5 = [dict(gamma=g, M=m / 1000.0, mu=mu) for g, m, mu in
       zip([1.4, 1.67, 1.3, 1.32, 1.4], [28.96, 4.0, 44.0, 16.0, 2.0],
           [1.8e-5, 1.99e-5, 1.47e-5, 1.1e-5, 0.88e-5])]


def cases():
    out = []
    out.append(("sod2d", abi.make_config(
        2, (24, 16), L=(1.0, 1.0), dt=1e-4, species=[dict(gamma=1.4, M=1.0, mu=2.928e-5)], R=1.0,
        ceq=True, kap=10.0, eps=0.4, alpha=40.0,
        bcs=("outflow", "outflow", "reflective", "reflective", "outflow", "outflow")),
        dict(kind=abi.IC_SHOCK_TUBE_2D, seed=1), 20))
    out.append(("rt2d", abi.make_config(
        2, (16, 24), L=(1.0 / 3.0, 1.0), dt=1e-4,
        species=[dict(gamma=1.4, M=1.0, mu=2.928e-5), dict(gamma=1.4, M=2.0, mu=2.928e-5)], R=1.0,
        visc=True, ceq=True, buoyancy=True, g=0.5, rho_ref=1.5, periodic=(True, False, False),
        bcs=("outflow", "outflow", "hydrostatic", "hydrostatic", "outflow", "outflow")),
        dict(kind=abi.IC_RT_2D, seed=7, rho_heavy=2.0, rho_light=1.0, p_ambient=2.4), 20))
    out.append(("smooth2d", abi.make_config(
        2, (13, 11), dt=2e-4, species=SP5[:3], R=1.0, visc=True,
        bcs=("noslip", "reflective", "hydrostatic", "outflow", "outflow", "outflow")),
        dict(kind=abi.IC_RANDOM_SMOOTH, seed=11), 10))
    out.append(("exp3d", abi.make_config(
        3, (8, 7, 6), dt=6e-5, species=[AIR, HE], visc=True, ceq=True, kap=10.0, eps=0.4,
        alpha=40.0),
        dict(kind=abi.IC_EXPANSION_3D, seed=20261203, p_ambient=1e5, T_ambient=300.0, p_high=1e7,
             radius=0.3, noise=0.01), 8))
    out.append(("mix3d", abi.make_config(
        3, (6, 7, 5), dt=2e-7, species=SP5, visc=True, ceq=True, buoyancy=True, g=9.81,
        rho_ref=1.0, periodic=(True, False, False),
        bcs=("outflow", "outflow", "hydrostatic", "noslip", "reflective", "outflow")),
        dict(kind=abi.IC_MIXING_3D, seed=20261206, p_ambient=1e5, T_ambient=300.0, nkernels=8), 8))
    out.append(("smooth3d", abi.make_config(
        3, (7, 6, 8), dt=2e-4, species=SP5[:3], R=1.0, visc=True, periodic=(False, False, True),
        bcs=("reflective", "noslip", "outflow", "hydrostatic", "outflow", "outflow")),
        dict(kind=abi.IC_RANDOM_SMOOTH, seed=13), 8))
    out.append(("smooth3d_ceq_per", abi.make_config(
        3, (6, 5, 7), dt=2e-4, species=SP5[:2], R=1.0, visc=True, ceq=True,
        periodic=(True, True, True)),
        dict(kind=abi.IC_RANDOM_SMOOTH, seed=17), 8))
    return out


def main():
    if not Reference.available():
        build_reference()
    for name, cfg, ic, steps in cases():
        icp = dict(ic)
        kind = icp.pop("kind")
        seed = icp.pop("seed")
        U0 = initial_conditions(cfg, kind, seed, **icp)
        r = Reference(cfg)
        r.set_state(U0)
        r.apply_bcs()
        R1 = r.compute_rhs()
        r = Reference(cfg)
        r.set_state(U0)
        r.rk_step(steps)
        UN = r.get_state()
        SN = r.secondary()
        meta = dict(name=name, config=abi.config_to_dict(cfg), ic=ic, steps=steps,
                    source="reference sources compiled by oracle/ref_build.sh")
        path = os.path.join(HERE, f"{name}.npz")
        np.savez_compressed(path, U0=U0, R1=R1, UN=UN, SN=SN, meta=json.dumps(meta))
        assert np.isfinite(UN).all() and np.isfinite(R1).all(), name
        print(f"{name}: {os.path.getsize(path) / 1024:.0f} KiB, |R1|max={np.abs(R1).max():.3g}")


if __name__ == "__main__":
    main()
