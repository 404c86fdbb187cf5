"""The oracle against golden vectors produced by the reference's own C++ (tests/golden)."""
import numpy as np

from conftest import rel_err


def test_raw_polynomials_match_reference(oracle_lib, golden):
    # x2o::poly_2b_v6x::eval / x2o::poly_3b_v2x::eval vs the monomial tables
    for body in ("2b", "3b"):
        X = golden["X" + body[0]]
        for k in range(len(X)):
            e, g = oracle_lib.poly(body, X[k])
            assert abs(e - golden["PE" + body][k]) <= 1e-13 * abs(golden["PE" + body][k])
            assert rel_err(g, golden["PG" + body][k]) <= 1e-13


def test_naive_and_trie_evaluators_agree(oracle_lib, golden):
    for body in ("2b", "3b"):
        for x in golden["X" + body[0]][:4]:
            e1, g1 = oracle_lib.poly(body, x)
            e2, g2 = oracle_lib.poly(body, x, naive=True)
            assert abs(e1 - e2) <= 1e-12 * abs(e1)
            assert rel_err(g1, g2) <= 1e-12


def test_2b_model_matches_reference(oracle_lib, golden):
    # tolerance: 1e-10 of max(|value|, 1 kcal/mol); the polynomial's own rounding is ~1e-11 absolute
    for k in range(len(golden["E2"])):
        e, g1, g2 = oracle_lib.model2b(golden["W2"][k, 0], golden["W2"][k, 1])
        ref = golden["E2"][k]
        assert abs(e - ref) <= 1e-10 * max(abs(ref), 1.0)
        g = np.concatenate([g1, g2])
        gr = golden["G2"][k].ravel()
        assert np.max(np.abs(g - gr)) <= 1e-10 * max(np.max(np.abs(gr)), 1.0)


def test_3b_model_matches_reference(oracle_lib, golden):
    for k in range(len(golden["E3"])):
        e, g1, g2, g3 = oracle_lib.model3b(*golden["W3"][k])
        ref = golden["E3"][k]
        assert abs(e - ref) <= 1e-10 * max(abs(ref), 1.0)
        g = np.concatenate([g1, g2, g3])
        gr = golden["G3"][k].ravel()
        assert np.max(np.abs(g - gr)) <= 1e-10 * max(np.max(np.abs(gr)), 1.0)


def test_golden_covers_switching_regimes(golden):
    W2 = golden["W2"]
    r = np.linalg.norm(W2[:, 0, :3] - W2[:, 1, :3], axis=1)
    assert (r < 4.5).any() and ((r > 4.5) & (r < 6.5)).any() and (r > 6.5).any()
    assert (golden["E2"][r > 6.5] == 0).all()
    assert (golden["E3"] == 0).any() and (golden["E3"] != 0).any()
