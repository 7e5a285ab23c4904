"""The engine's own table builder (pi-qmc_gb300/csrc/tables.cc), used when the
engine runs standalone: CoulombAction pair tables against the tables pi-qmc
built (golden fixtures), and the OptEwaldSum long-range table against pi-qmc's
own system-test expectation, the NaCl Madelung energy
(test/system/madelung/test_nacl.py:21-37, -1.747564594633182 per ion pair, 1e-5)."""
import numpy as np
import pytest

import golden_io


@pytest.fixture(scope="module")
def pimc():
    import pimc_gb300
    pimc_gb300.build.build()
    return pimc_gb300


@pytest.mark.parametrize("case", ["dot2_full", "dot20_fn"])
def test_coulomb_pair_tables_match_reference(pimc, case):
    g = golden_io.load(case)
    tabs, ew = pimc.coulomb_tables(g["kw"])
    assert ew is None
    assert len(tabs) == len(g["tables"])
    for t, r in zip(tabs, g["tables"]):
        assert tuple(t["species"]) == tuple(r["species"])
        assert t["rgridinv"] == r["rgridinv"] and t["logrratioinv"] == r["logrratioinv"]
        u, ur = t["ugrid"][:, 0], r["ugrid"][:, 0]
        assert np.all(np.abs(u - ur) <= 1e-13 * np.maximum(np.abs(ur), 1e-3))
        # the tau derivative is a central difference with step 1e-7 tau in both
        # codes, which turns rounding of u into ~1e-8 relative noise
        ut, utr = t["ugrid"][:, 1], r["ugrid"][:, 1]
        assert np.all(np.abs(ut - utr) <= 1e-6 * np.maximum(np.abs(utr), 1e-3))


def test_ewald_kvectors_match_reference(pimc):
    g = golden_io.load("heg54")
    tabs, ew = pimc.coulomb_tables(g["kw"])
    assert ew["totk"] == g["ewald"]["totk"] == 257
    assert np.array_equal(ew["kvec"], g["ewald"]["kvec"])
    assert ew["ikmax"] == g["ewald"]["ikmax"]
    assert ew["one_over_2v"] == g["ewald"]["one_over_2v"]


def test_nacl_madelung_energy(pimc):
    # test/system/madelung/pimc.xml: a=2 cell, 4 Na+ and 4 Cl-, rcut 0.5, kcut 50.
    kw = dict(counts=[4, 4], masses=[41920.0, 63800.0], charges=[1.0, -1.0], nslice=10,
              beta=1.0, nlevel=1, coulomb=1, ewald=1, ewald_kcut=50.0, cell=2.0)
    tabs, ew = pimc.coulomb_tables(kw, norder=1, ngpts=1000, rmin=0.01, rmax=3.0,
                                   ewald_rcut=0.5)
    pos = np.array([[0, 0, 0], [1, 1, 0], [1, 0, 1], [0, 1, 1],
                    [1, 0, 0], [0, 1, 0], [0, 0, 1], [1, 1, 1]], float)
    q = np.array([1, 1, 1, 1, -1, -1, -1, -1.0])
    k = ew["kvec"] * (2 * 3.14159265358979 / 2.0)
    rho = (q[None, :] * np.exp(1j * (k @ pos.T))).sum(1)
    # all ion pairs are farther apart than rcut: the energy is the k-space sum
    e = (2 * ew["vk"] * np.abs(rho) ** 2).sum() * ew["one_over_2v"] + ew["self_energy"]
    assert e / 4 == pytest.approx(-1.747564594633182, abs=1e-5)


@pytest.mark.parametrize("case", ["heg8", "heg54", "heg16_hot"])
def test_action_ewald_table_against_reference(pimc, case):
    # The long-range table the engine's own builder fits for CoulombAction
    # (OptEwaldSum's constrained least squares, solved as one KKT system in the
    # scaled basis (r/rc)^2n) against the table pi-qmc's OptEwaldSum built for the
    # same system (golden fixture).  pi-qmc forms the normal equations in the
    # monomial basis (condition number ~2e32 for these boxes), so its
    # coefficients are set by rounding to ~1e-3; the two fits agree on the
    # k-list, 1/(2V) and ikmax exactly, on v_k to 5e-3 of max |v_k| and on the
    # self energy to 1e-3 relative.
    g = golden_io.load(case)
    tabs, ew = pimc.coulomb_tables(g["kw"])
    r = g["ewald"]
    assert ew["totk"] == r["totk"] and np.array_equal(ew["kvec"], r["kvec"])
    assert ew["ikmax"] == r["ikmax"] and ew["one_over_2v"] == r["one_over_2v"]
    assert np.max(np.abs(ew["vk"] - r["vk"])) <= 5e-3 * np.abs(r["vk"]).max()
    assert ew["self_energy"] == pytest.approx(r["self_energy"], rel=1e-3)
