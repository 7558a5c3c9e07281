"""Skyrme residual-interaction couplings for the charge-changing (T=1) channel.

Follows pnfam_interaction.f90: ``init_interaction`` (:90-261) turns the
namelist ``&interaction`` and the HFB functional into the coupling constants
used by the density -> field step, with the density-dependent ones tabulated
on the mesh: C^rho(r) = C^rho_0 + C^rho_r rho^sigma, C^s(r), and the pairing
couplings C^pair(r), C^spair(r) (:246-258).  The Skyrme (t, x) -> C
conversion is the one at :669-690; gauge-invariance fixing at :121-124.

The parameter sets below are the published values of each functional
(the citations are the functionals' own papers).
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

HUGE = np.finfo(float).max


class InteractionError(RuntimeError):
    pass


# name -> (label, t0, t1, t2, t3, x0, x1, x2, x3, b4, b4p, alpha, tte, tto, uses_j2); the
# parameter sets the reference tabulates (pnfam_interaction.f90:339-667), with the spin-orbit
# b4 = b4' = W0/2 where a set gives W0.  The same numbers are needed to give the same
# couplings; the papers are those the reference cites:
# SIII: M. Beiner et al., Nucl. Phys. A 238, 29 (1975) (HFBTHO v2 alpha and x3)
# SGII: N. V. Giai, H. Sagawa, Phys. Lett. B 106, 379 (1981)
# SkM*: J. Bartel et al., Nucl. Phys. A 386, 79 (1982)
# SkO, SkO': P.-G. Reinhard et al., Phys. Rev. C 60, 014316 (1999)
# SLy4, SLy5: E. Chabanat et al., Nucl. Phys. A 635, 231 (1998) (HFBTHO's rounding, and the
#   published values as SLY4PUB / SLY5PUB)
# T43: T. Lesinski et al., Phys. Rev. C 76, 014312 (2007)
# SV-min: P. Kluepfel et al., Phys. Rev. C 79, 034310 (2009)
# UNEDF0/1/2: M. Kortelainen et al., Phys. Rev. C 89, 054314 (2014) supplement (tensor terms
#   dropped for UNEDF0/1, as in the reference); UNEDF1-HFB: N. Schunck et al., J. Phys. G 42,
#   034024 (2015) (time-odd tensor terms dropped)
_SKYRME = {
    "SIII": ("SIII", -1128.75, 395.0, -95.0, 14000.0, 0.45, 0.0, 0.0, 1.0,
             120.0 / 2.0, 120.0 / 2.0, 1.0, 0.0, 0.0, False),
    "SGII": ("SGII", -2645.0, 340.0, -41.9, 15595.0, 0.09, -0.0588, 1.425, 0.06044,
             105.0 / 2.0, 105.0 / 2.0, 1.0 / 6.0, 0.0, 0.0, False),
    "SKM*": ("SkM*", -2645.0, 410.0, -135.0, 15595.0, 0.09, 0.0, 0.0, 0.0,
             65.0, 65.0, 1.0 / 6.0, 0.0, 0.0, False),
    "SKO": ("SkO", -2103.653, 303.352, 791.674, 13553.252, -0.210701, -2.810752, -1.461595,
            -0.429881, 176.578, -198.7490, 1.0 / 4.0, 0.0, 0.0, False),
    "SKOP": ("SkO'", -2099.419, 301.531, 154.781, 13526.464, -0.029503, -1.325732,
             -2.323439, -0.147404, 143.895, -82.8888, 0.25, 0.0, 0.0, True),
    "SLY4": ("SLy4", -2488.913, 486.818, -546.395, 13777.0, 0.834, -0.344, -1.0, 1.354,
             61.5, 61.5, 1.0 / 6.0, 0.0, 0.0, False),
    "SLY4PUB": ("SLy4 (published)", -2488.91, 486.820, -546.390, 13777.0, 0.834, -0.344, -1.000, 1.354,
                123.0 / 2.0, 123.0 / 2.0, 1.0 / 6.0, 0.0, 0.0, False),
    "SLY5": ("SLy5 (HFBTHO)", -2483.45, 484.23, -556.69, 13757.00, 0.776, -0.317, -1.000, 1.263,
             125.0 / 2.0, 125.0 / 2.0, 1.0 / 6.0, 0.0, 0.0, True),
    "SLY5PUB": ("SLy5 (published)", -2484.88, 483.13, -549.40, 13763.00, 0.778, -0.328, -1.000, 1.267,
                126.0 / 2.0, 126.0 / 2.0, 1.0 / 6.0, 0.0, 0.0, True),
    "T43": ("T43", -2490.275, 494.608, -255.534, 13847.12, 0.698702, -0.781655, -0.646302, 1.135795,
            153.103 / 2.0, 153.103 / 2.0, 1.0 / 6.0, 196.868, -49.160, True),
    "SVMIN": ("SV-min", -2112.248, 295.781, 142.268, 13988.567, 0.243886, -1.434926, -2.625899,
              0.258070, 111.291 / 2.0, 45.93615, 0.255368, 0.0, 0.0, False),
    "UNEDF0": ("UNEDF0", -1883.68781034247695, 277.500212238931113, 608.430905591534383,
               13901.9483446343256, 0.00974374651612197606, -1.77784394560870229,
               -1.67699034528797575, -0.380790414633100260, 125.161, -91.2604,
               0.321955989588264435, 0.0, 0.0, False),
    "UNEDF1": ("UNEDF1", -2078.32802325564080, 239.400812041522045, 1575.11954189757989,
               14263.6462470775950, 0.0537569206858470316, -5.07723238187693671,
               -1.36650561394298609, -0.162491168089956339, 38.3680720616682009, 71.3165222295833985,
               0.270018011502707600, 0.0, 0.0, False),
    "UNEDF2": ("UNEDF2", -1735.45685190850349, 262.814456235313969, 1183.31263243304011,
               12293.2432941125371, 0.172247227624101162, -3.76692685046941023,
               -1.38349812677880979, 0.0528642727436126059, 25.6586677306483040, 77.3003893702710059,
               0.351455132555483607, -240.140598215558754, -266.930662318713644, True),
    "UNEDF1-HFB": ("UNEDF1-HFB", -1666.40609652204898, 255.225795498529067, 1521.27603913447047,
                   12072.5070586946749, 0.146079699879160696, -4.82248258717499834,
                   -1.35211044158474336, 0.00431668727902556615, 22.0338399999999979, 103.825096000000002,
                   0.376580313583912030, 0.0, 0.0, False),
}
_ALIASES = {"SKO'": "SKOP", "S3": "SIII", "SG2": "SGII", "SV-MIN": "SVMIN", "UNE0": "UNEDF0",
            "UNE1": "UNEDF1", "UNE2": "UNEDF2", "UNEDF1HFB": "UNEDF1-HFB", "UNE1HFB": "UNEDF1-HFB",
            "UNE1-HFB": "UNEDF1-HFB", "HFB1": "UNEDF1-HFB"}


@dataclass
class Couplings:
    """Coupling constants of the residual interaction (names as in the reference)."""
    name: str = "NONE"
    skip_residual_interaction: bool = True
    cr0: float = 0.0
    crr: float = 0.0
    cs0: float = 0.0
    csr: float = 0.0
    sigma_r: float = 0.0
    sigma_s: float = 0.0
    cpair0: float = 0.0
    cpairr: float = 0.0
    cspair0: float = 0.0
    cspairr: float = 0.0
    sigma_pair: float = 0.0
    cdrho: float = 0.0
    ctau: float = 0.0
    ctj0: float = 0.0
    ctj1: float = 0.0
    ctj2: float = 0.0
    crdj: float = 0.0
    cds: float = 0.0
    ct: float = 0.0
    cj: float = 0.0
    cgs: float = 0.0
    cf: float = 0.0
    csdj: float = 0.0
    crho: np.ndarray = field(default=None)    # [nghl]
    cs: np.ndarray = field(default=None)
    cpair: np.ndarray = field(default=None)
    cspair: np.ndarray = field(default=None)

    def scalars(self) -> np.ndarray:
        """The 12 mesh-independent couplings in the order the kernels expect:
        cdrho, ctau, ctj0, ctj1, ctj2, crdj, cds, ct, cj, cgs, cf, csdj."""
        return np.array([self.cdrho, self.ctau, self.ctj0, self.ctj1, self.ctj2, self.crdj,
                         self.cds, self.ct, self.cj, self.cgs, self.cf, self.csdj], dtype=np.float64)


def _skyrme_to_couplings(c: Couplings, p):
    (_, t0, t1, t2, t3, x0, x1, x2, x3, b4, b4p, alpha, tte, tto, uses_j2) = p
    c.cr0 = -1.0 / 8.0 * t0 * (2.0 * x0 + 1.0)
    c.crr = -1.0 / 48.0 * t3 * (2.0 * x3 + 1.0)
    c.cs0 = -1.0 / 8.0 * t0
    c.csr = -1.0 / 48.0 * t3
    c.sigma_r = alpha
    c.sigma_s = alpha
    c.cdrho = 3.0 / 32.0 * t1 * (x1 + 0.5) + 1.0 / 32.0 * t2 * (x2 + 0.5)
    c.ctau = -1.0 / 8.0 * t1 * (x1 + 0.5) + 1.0 / 8.0 * t2 * (x2 + 0.5)
    c.ctj0 = 1.0 / 48.0 * (t1 - t2 + 10.0 * tte - 10.0 * tto)
    c.ctj1 = 1.0 / 32.0 * (t1 - t2 - 5.0 * tte + 5.0 * tto)
    c.ctj2 = 1.0 / 16.0 * (t1 - t2 + tte - tto)
    c.crdj = -0.5 * b4p
    c.cds = 1.0 / 64.0 * (3.0 * t1 + t2 - 6.0 * tte - 2.0 * tto)
    c.ct = -1.0 / 16.0 * (t1 - t2 - 2.0 * tte + 2.0 * tto)
    c.cj = 1.0 / 8.0 * t1 * (x1 + 0.5) - 1.0 / 8.0 * t2 * (x2 + 0.5)
    c.cgs = -3.0 / 32.0 * (3.0 * tte + tto)
    c.cf = -3.0 / 8.0 * (tte - tto)
    c.csdj = -0.5 * b4p
    # extended tensor terms are not used by these sets
    c.ctj0 = 2.0 / 3.0 * c.ctj1
    c.ctj2 = 2.0 * c.ctj1
    return uses_j2


def _read_custom(path: str, c: Couplings):
    from .namelist import parse_namelist_file
    groups = parse_namelist_file(path)
    g = groups.get("custom_interaction")
    if g is None:
        raise InteractionError(f'could not read interaction file "{path}"')
    for k, v in g.items():
        if hasattr(c, k):
            setattr(c, k, float(v))


def init_interaction(nml: dict, hfb, rho_total: np.ndarray) -> Couplings:
    """Build the couplings from the ``&interaction`` namelist group ``nml`` and
    the HFB solution (its pairing functional and saturation density)."""
    c = Couplings()
    name = str(nml.get("interaction_name", "NONE")).strip()
    uname = name.upper()
    h = hfb.hel
    if uname == "NONE":
        c.skip_residual_interaction = True
        n = len(rho_total)
        c.crho = np.zeros(n); c.cs = np.zeros(n); c.cpair = np.zeros(n); c.cspair = np.zeros(n)
        return c
    c.skip_residual_interaction = False
    if uname.startswith("FILE:"):
        _read_custom(name[5:].strip(), c)
        c.name = name
    else:
        key = _ALIASES.get(uname, uname)
        if key not in _SKYRME:
            raise InteractionError(f'interaction "{name}" not found.')
        p = _SKYRME[key]
        c.name = p[0]
        uses_j2 = _skyrme_to_couplings(c, p)
        if not uses_j2 and not bool(nml.get("force_j2_terms", False)):
            c.ctj0 = c.ctj1 = c.ctj2 = 0.0
        if bool(nml.get("require_gauge_invariance", False)):
            c.cf = 2 * c.ctj1 - c.ctj2
            c.ct = -2 * c.ctj1 + 0.5 * c.cf
        rho_c = float(h.nm[3])
        vpair_t0 = nml.get("vpair_t0", None)
        vpair0 = nml.get("vpair0", None)
        vpair_t1 = nml.get("vpair_t1", None)
        vpair1 = nml.get("vpair1", None)
        if vpair_t0 is None:
            vpair_t0 = 0.0 if vpair0 is None else 2 * float(vpair0)
        elif vpair0 is not None:
            raise InteractionError("cannot set both vpair0 and vpair_t0!")
        if vpair_t1 is None:
            vpair_t1 = 0.5 * float(np.sum(h.CpV0)) if vpair1 is None else float(vpair1)
        elif vpair1 is not None:
            raise InteractionError("cannot set both vpair1 and vpair_t1!")
        if abs(c.sigma_pair) < np.finfo(np.float32).eps:
            c.sigma_pair = 1.0
        c.cpair0 = float(vpair_t1) / 8.0
        c.cspair0 = float(vpair_t0) / 8.0
        c.cpairr = c.cpair0 * (-1.0 * h.CpV1[0] / rho_c ** c.sigma_pair)
        c.cspairr = c.cspair0 * (-1.0 * h.CpV1[0] / rho_c ** c.sigma_pair)
        for key_o, attr in (("override_cs0", "cs0"), ("override_csr", "csr"), ("override_cds", "cds"),
                            ("override_ct", "ct"), ("override_cf", "cf"), ("override_cgs", "cgs"),
                            ("override_cj", "cj"), ("override_csdj", "csdj")):
            v = nml.get(key_o, None)
            if v is not None:
                setattr(c, attr, float(v))
        if bool(nml.get("require_self_consistency", True)):
            _check_self_consistency(c, h, rho_c)
    rho = rho_total
    c.crho = c.cr0 + c.crr * rho ** c.sigma_r
    c.cs = c.cs0 + c.csr * rho ** c.sigma_s
    c.cpair = c.cpair0 + c.cpairr * rho ** c.sigma_pair
    c.cspair = c.cspair0 + c.cspairr * rho ** c.sigma_pair
    return c


def _check_self_consistency(c: Couplings, h, rho_c: float, tol: float = 5.0e-12):
    """check_self_consistency (pnfam_interaction.f90:820-925): abort when the
    residual interaction does not match the functional of the ground state."""
    bad = []
    if abs(h.Crho[1] - c.cr0) > tol: bad.append("Crho[0]")
    if abs(h.Cdrho[1] - c.crr) > tol: bad.append("Crho[r]")
    if abs(h.CrDr[1] - c.cdrho) > tol: bad.append("Cdrho")
    if abs(h.Ctau[1] - c.ctau) > tol: bad.append("Ctau")
    if not h.use_j2terms:
        if abs(c.ctj1) > tol: bad.append("CJ1")
    else:
        if abs(h.CJ[1] - 2 * c.ctj1) > tol: bad.append("CJ1")
        if abs(h.CJ[1] - c.ctj2) > tol: bad.append("CJ2")
    if abs(h.CrdJ[1] - c.crdj) > tol: bad.append("CrdJ")
    if abs(0.5 * float(np.sum(h.CpV0)) - 8 * c.cpair0) > tol: bad.append("Cpair")
    if bad:
        raise InteractionError("this is not a self-consistent calculation: " + ", ".join(bad))
