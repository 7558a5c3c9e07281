"""Set-up of one pnFAM calculation: namelist -> ground state, couplings, operator.

Mirrors setup_pnfam (pnfam_setup.f90:152-192), setup_extfield
(pnfam_solver.f90:556-654, one-body part) and the Broyden mixing constant
(pnfam_broyden.f90:20).  Two-body-current modes are not supported
(two_body_current_mode must be 0).
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from .extfield import ExternalField, init_external_field, setup_crossterms
from .hfb_solution import HFBSolution, load_hfb_solution
from .interaction import Couplings, init_interaction

# pnfam_broyden.f90:20 initialises the mixing factor from the default-real
# literal 0.7, i.e. the float32 value 0.699999988079071044921875.
ALPHA_MIX = float(np.float32(0.7))


class SetupError(RuntimeError):
    pass


@dataclass
class Case:
    hfb: HFBSolution
    couplings: Couplings
    F: ExternalField
    G: list
    nml: dict

    @property
    def omega(self) -> complex:
        g = self.nml["general"]
        return complex(float(g["real_eqrpa"]), float(g["imag_eqrpa"]))

    @property
    def quench(self) -> float:
        q = float(self.nml["solver"]["quench_residual_int"])
        return 0.0 if self.couplings.skip_residual_interaction else q


def setup_case(nml: dict, hel_path: str, hfb: HFBSolution = None) -> Case:
    e = nml["ext_field"]
    if int(e.get("two_body_current_mode", 0)) != 0:
        raise SetupError("two_body_current_mode /= 0 is not supported by this solver")
    if hfb is None:
        hfb = load_hfb_solution(hel_path)
    s = nml["solver"]
    if float(s["energy_shift_prot"]) != 0.0 or float(s["energy_shift_neut"]) != 0.0:
        hfb = _shifted(hfb, float(s["energy_shift_prot"]), float(s["energy_shift_neut"]))
    cp = init_interaction(nml["interaction"], hfb, hfb.rho_n + hfb.rho_p)
    F = init_external_field(hfb, e["beta_type"], e["operator_name"], int(e["operator_k"]))
    G = setup_crossterms(hfb, F) if bool(e["compute_crossterms"]) else []
    return Case(hfb, cp, F, G, nml)


def _shifted(hfb: HFBSolution, dp: float, dn: float) -> HFBSolution:
    """Ep = Epe + energy_shift_prot, En = Ene + energy_shift_neut (pnfam_setup.f90:316-317)."""
    import copy
    h = copy.copy(hfb)
    h.Ep = hfb.Ep + dp
    h.En = hfb.En + dn
    return h
