"""Set-up of one pnFAM calculation: namelist -> ground state, couplings, operator.

Mirrors setup_pnfam (pnfam_setup.f90:152-192), setup_extfield
(pnfam_solver.f90:556-654, with the two-body-current modes) and the Broyden
mixing constant (pnfam_broyden.f90:20).
"""
from __future__ import annotations

import os
from dataclasses import dataclass

import numpy as np

from .extfield import ExternalField, init_external_field, setup_crossterms
from .extfield_2bc import LECs, TwoBodyCurrentError, finite_range_field, parse_mode
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


def setup_case(nml: dict, hel_path: str, hfb: HFBSolution = None, tbc_dir: str = ".",
               twobc_revision: dict = None) -> Case:
    """``tbc_dir``: where ``<fam_output_filename>.tbc`` (the cached finite-range
    two-body-current field) is looked up, the working directory of pnfam_main;
    ``twobc_revision``: overrides of the hard-coded two-body-current constants
    (``extfield_2bc.LECs``), to reproduce runs of earlier reference revisions."""
    e = nml["ext_field"]
    if hfb is None:
        hfb = load_hfb_solution(hel_path)
    s = nml["solver"]
    if float(s["energy_shift_prot"]) != 0.0 or float(s["energy_shift_neut"]) != 0.0:
        hfb = _shifted(hfb, float(s["energy_shift_prot"]), float(s["energy_shift_neut"]))
    cp = init_interaction(nml["interaction"], hfb, hfb.rho_n + hfb.rho_p)
    mode = int(e.get("two_body_current_mode", 0) or 0)
    try:
        use_2bc = parse_mode(mode)
        lecs = LECs.from_namelist(e.get("two_body_current_lecs", [-3.4, 5.4, 0.0]),
                                  bool(e.get("two_body_current_usep", False)),
                                  **(twobc_revision or {})) if mode else None
        F, G = _external_field(hfb, e, use_2bc, lecs, nml["general"].get("fam_output_filename", ""), tbc_dir)
    except TwoBodyCurrentError as err:
        raise SetupError(str(err))
    return Case(hfb, cp, F, G, nml)


def _external_field(hfb, e, use_2bc, lecs, out_name, tbc_dir):
    """setup_extfield (pnfam_solver.f90:556-654)."""
    label = str(e["operator_name"]).strip().upper()
    k = int(e["operator_k"])
    beta = e["beta_type"]
    direct_2bc = label in ("P", "PS0", "RS0", "RS1", "RS2", "RS0I", "RS1I") and any(use_2bc)
    F = init_external_field(hfb, beta, label, k, use_2bc if direct_2bc else (0,) * 6, lecs)
    G = setup_crossterms(hfb, F, use_2bc, lecs) if bool(e["compute_crossterms"]) else []
    if label != "GT" or not any(use_2bc) or use_2bc[3] == 0:
        return F, G
    # GT: -sigma tau (Park sign convention, 1+2 body) + contact/LDA/DME part ...
    tmp = -F.mat.flatten() if use_2bc[0] == 1 else np.zeros(F.mat.nelem)
    contact = init_external_field(hfb, beta, label, k, use_2bc, lecs)
    tmp = tmp + contact.mat.flatten()
    if use_2bc[1] not in (1, 5):
        F.mat.set_flat(tmp)
        return F, G
    # ... + the finite-range part (direct only with the DME exchange form)
    path = os.path.join(tbc_dir, f"{str(out_name).strip()}.tbc")
    mode = int(e.get("two_body_current_mode", 0) or 0)
    fr = finite_range_field(path, hfb, F, lecs, lecs.use_p, use_2bc[1] == 5, mode, len(G))
    F.mat.set_flat(fr + tmp)
    return F, G


def _shifted(hfb: HFBSolution, dp: float, dn: float) -> HFBSolution:
    """Ep = Epe + energy_shift_prot, En = Ene + energy_shift_neut (pnfam_setup.f90:316-317)."""
    import copy
    h = copy.copy(hfb)
    h.Ep = hfb.Ep + dp
    h.En = hfb.En + dn
    return h
