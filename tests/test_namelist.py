import pytest

from pynfam_gb300.namelist import NamelistError, parse_namelist_text, read_pnfam_namelist

TEXT = """&general
    fam_output_filename = 'GT-K0'
    print_stdout = .true.
    real_eqrpa = 1.5e-05
    imag_eqrpa = -0.0129
/

&ext_field
    beta_type = '-'
    operator_name = 'gt'
    operator_k = 1
    compute_crossterms = T
    two_body_current_lecs = -3.1962, 3.1962, 0
/

&interaction
    interaction_name = 'SKOP'
    vpair_t0 = -346.352
    vpair_t1 = ,
    override_cs0 = 128.279d0
/

&solver
    max_iter = 300
    convergence_epsilon = 1e-07
/
"""


def test_parse_groups(tmp_path):
    p = tmp_path / "OP.in"
    p.write_text(TEXT)
    n = read_pnfam_namelist(str(p))
    assert n["general"]["fam_output_filename"] == "GT-K0"
    assert n["general"]["imag_eqrpa"] == -0.0129
    assert n["ext_field"]["operator_name"] == "GT" and n["ext_field"]["operator_k"] == 1
    assert n["ext_field"]["compute_crossterms"] is True
    assert n["ext_field"]["two_body_current_lecs"] == [-3.1962, 3.1962, 0]
    assert n["interaction"]["vpair_t0"] == -346.352
    assert n["interaction"]["vpair_t1"] is None          # empty value keeps the default
    assert n["interaction"]["override_cs0"] == 128.279
    assert n["solver"]["max_iter"] == 300
    assert n["solver"]["broyden_history_size"] == 50     # default


def test_unknown_entry_is_an_error(tmp_path):
    p = tmp_path / "OP.in"
    p.write_text("&solver\n  no_such_thing = 1\n/\n")
    with pytest.raises(NamelistError):
        read_pnfam_namelist(str(p))


def test_missing_file():
    with pytest.raises(NamelistError):
        read_pnfam_namelist("/nonexistent/OP.in")


def test_unterminated_group():
    with pytest.raises(NamelistError):
        parse_namelist_text("&solver\n max_iter = 3\n")


def test_every_tabulated_functional_gives_couplings():
    """Each Skyrme set the reference tabulates (and its aliases) builds finite couplings on a
    recorded ground state (pnfam_interaction.f90:339-690); the tensor-free relation
    CJ0 = 2/3 CJ1, CJ2 = 2 CJ1 holds (:704-708)."""
    import numpy as np
    from golden_cases import hfb
    from pynfam_gb300.interaction import _ALIASES, _SKYRME, init_interaction
    h = hfb("S40")
    for name in list(_SKYRME) + list(_ALIASES):
        nml = {"interaction_name": name, "require_self_consistency": False, "require_gauge_invariance": False,
               "force_j2_terms": False}
        c = init_interaction(nml, h, h.rho_n + h.rho_p)
        assert not c.skip_residual_interaction
        assert np.all(np.isfinite(c.crho)) and np.all(np.isfinite(c.scalars()))
        assert abs(c.ctj0 - 2.0 / 3.0 * c.ctj1) < 1e-12 and abs(c.ctj2 - 2.0 * c.ctj1) < 1e-12
