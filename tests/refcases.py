"""Golden vectors computed by the reference's own source (tests/golden/ref,
made by tests/golden/make_ref_fixtures.py) and the same setups as a
CaseConfig (read by CaseConfig.from_setups, the product's own reader) and as an
oracle case."""
import glob
import json
import os

import numpy as np
import torch

from oracle import jf_oracle as O

REF_DIR = os.path.join(os.path.dirname(__file__), "golden", "ref")


def names():
    return sorted(os.path.splitext(os.path.basename(p))[0] for p in glob.glob(os.path.join(REF_DIR, "*.npz")))


def load(name):
    with np.load(os.path.join(REF_DIR, f"{name}.npz")) as z:
        fx = {k: z[k] for k in z.files}
    fx["case_setup"] = json.loads(str(fx["case_setup"]))
    fx["numerical_setup"] = json.loads(str(fx["numerical_setup"]))
    fx["steps"] = int(fx["steps"])
    fx["t"] = float(fx["t"])
    return fx


def configs(fx):
    """(OracleCase, CaseConfig) of a fixture's setups."""
    from jaxfluids_gb300.config import CaseConfig
    cc = CaseConfig.from_setups(fx["case_setup"], fx["numerical_setup"])
    oc = O.OracleCase(
        cells=cc.cells, ranges=cc.ranges, nh=cc.nh, gamma=cc.gamma, R=cc.R,
        bc={f: cc.bc.get(f, "INACTIVE") for f in O.FACES}, recon=cc.recon, recon_var=cc.recon_var,
        frozen_state=cc.frozen_state, riemann=cc.riemann, signal_speed=cc.signal_speed, cfl=cc.cfl,
        fixed_dt=cc.fixed_dt, viscous=cc.viscous, heat=cc.heat, mu=cc.mu, bulk_viscosity=cc.bulk_viscosity,
        thermal_conductivity=cc.kappa if cc.heat else None, viscous_heat_production=cc.viscous_heat_production,
        bc_values=dict(cc.bc_values), diss_recon=cc.diss_recon, diss_deriv_center=cc.diss_deriv_center,
        diss_deriv_face=cc.diss_deriv_face, convective=cc.convective)
    return oc, cc


def prims0(fx):
    return torch.from_numpy(np.ascontiguousarray(fx["prims0"]))


def rel_diff(a, b):
    """max over variables of ||a_v - b_v||_inf / ||b_v||_inf (b the reference)."""
    a = np.asarray(a, dtype=np.float64).reshape(a.shape[0], -1)
    b = np.asarray(b, dtype=np.float64).reshape(b.shape[0], -1)
    worst = 0.0
    for v in range(a.shape[0]):
        den = np.abs(b[v]).max()
        num = np.abs(a[v] - b[v]).max()
        worst = max(worst, num / den if den > 0 else num)
    return worst
