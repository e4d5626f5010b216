"""The CPU restatement (oracle/) pinned against the reference's golden vectors."""
import numpy as np
import pytest

from golden_cases import CASES, adversarial, load


@pytest.mark.parametrize("name", CASES)
def test_restated_oracle_matches_reference_labels(orc, name):
    c = load(name)
    for v in range(len(c["eps"])):
        lab = orc.dbscan(c["x"], c["y"], c["eps"][v], c["minpts"][v], int(c["mbb"]))
        np.testing.assert_array_equal(lab, c["labels"][v], err_msg=f"{name} variant {v}")


def test_reference_test_output_csv(orc):
    # src/test_output.csv: columns label(eps=1,mp=10), label(eps=0.5,mp=12)
    c = load("reference_test_dataset")
    assert c["labels"].shape == (2, 225)
    # on this dataset the reference's reuse path equals the standalone path
    np.testing.assert_array_equal(c["multi"], c["labels"])


def test_vtest_known_answer(orc):
    # src/vtest.py: (3,3),(2,2),(8,8),(1,1); eps = sqrt(2) +- 0.01, minpts 2
    c = load("vtest")
    np.testing.assert_array_equal(c["labels"].T, [[1, 0], [1, 0], [0, 0], [1, 0]])
    got = np.stack([orc.dbscan(c["x"], c["y"], e, 2) for e in c["eps"]]).T
    np.testing.assert_array_equal(got, [[1, 0], [1, 0], [0, 0], [1, 0]])


def test_adversarial_asymmetric_cases(orc):
    cases = adversarial()
    assert len(cases) >= 20
    for i, c in enumerate(cases):
        lab = orc.dbscan(c["x"], c["y"], c["eps"], c["minpts"], c["mbb"])
        np.testing.assert_array_equal(lab, c["labels"], err_msg=f"case {i}")


@pytest.mark.parametrize("name,mbb", [("lattice_4k", 70), ("lattice_4k_mbb1", 1),
                                      ("edge_negative_dupes", 70)])
def test_grid_candidates_complete_vs_bruteforce(orc, name, mbb):
    c = load(name)
    for e in c["eps"]:
        g = orc.neighbor_counts(c["x"], c["y"], e, mbb)
        b = orc.neighbor_counts(c["x"], c["y"], e, mbb, bruteforce=True)
        np.testing.assert_array_equal(g, b)


def test_eps_threshold_is_tight(orc):
    for eps in [0.05, 0.1, 0.25, 0.5, 0.8, 1.0, np.sqrt(2) + 0.01, 1e-300, 3.7e5]:
        t = orc.eps_threshold(eps)
        assert np.sqrt(t) <= eps
        assert np.sqrt(np.nextafter(t, np.inf)) > eps
    assert orc.eps_threshold(-1.0) < 0
    assert orc.eps_threshold(0.0) == 0.0


def test_visit_order_is_stable_bin_sort(orc):
    c = load("single_variant_3k")
    m = orc.visit_order(c["x"], c["y"])
    assert sorted(m.tolist()) == list(range(3000))


def _mix64(v):
    # splitmix64 finaliser on uint64 arrays (wrapping arithmetic)
    v = v.astype(np.uint64)
    v ^= v >> np.uint64(30)
    v *= np.uint64(0xbf58476d1ce4e5b9)
    v ^= v >> np.uint64(27)
    v *= np.uint64(0x94d049bb133111eb)
    v ^= v >> np.uint64(31)
    return v


def _hash_from_lists(off, nb):
    # the table hash restated from the oracle's neighbour lists
    n = len(off) - 1
    p = np.repeat(np.arange(n, dtype=np.uint64), np.diff(off).astype(np.int64))
    q = nb.astype(np.uint64)
    fwd = (p << np.uint64(32)) | q
    back = (q << np.uint64(32)) | p
    oneway = ~np.isin(back, fwd)
    with np.errstate(over="ignore"):
        h = _mix64(fwd).sum(dtype=np.uint64)
        h += np.uint64(0x9e3779b97f4a7c15) * np.uint64(int(oneway.sum()))
    return int(h)


@pytest.mark.parametrize("name,mbb", [("lattice_4k", 70), ("lattice_4k_mbb1", 1),
                                      ("variant_sweep_4k", 70)])
def test_table_hash_restates_the_neighbour_lists(orc, name, mbb):
    c = load(name)
    for e in np.unique(c["eps"]):
        off, nb = orc.neighbor_lists(c["x"], c["y"], e, mbb)
        assert orc.table_hash(c["x"], c["y"], e, mbb) == _hash_from_lists(off, nb)


def test_table_hash_sees_one_way_pairs(orc):
    # the adversarial cases hold pairs accepted in one direction only
    seen = 0
    for c in adversarial():
        off, nb = orc.neighbor_lists(c["x"], c["y"], c["eps"], c["mbb"])
        h = orc.table_hash(c["x"], c["y"], c["eps"], c["mbb"])
        assert h == _hash_from_lists(off, nb)
        n = len(off) - 1
        p = np.repeat(np.arange(n), np.diff(off).astype(np.int64))
        fwd = set(zip(p.tolist(), nb.tolist()))
        seen += sum((q, pp) not in fwd for pp, q in fwd)
    assert seen > 0


def test_many_variants_equal_one_at_a_time(orc):
    # orc_dbscan_many (counts shared per epsilon, variants in parallel
    # threads) gives each variant the labels of its own orc_dbscan call,
    # repeated and NaN epsilons included
    from golden_cases import load as load_case
    for name in ("variant_sweep_4k", "lattice_4k", "reference_test_dataset"):
        c = load_case(name)
        eps = np.concatenate([c["eps"], [c["eps"][0], np.nan]])
        mp = np.concatenate([c["minpts"], [3, 4]]).astype(np.uint32)
        many = orc.variants(c["x"], c["y"], eps, mp, int(c["mbb"]))
        for v in range(len(eps)):
            one = orc.dbscan(c["x"], c["y"], eps[v], mp[v], int(c["mbb"]))
            np.testing.assert_array_equal(many[v], one, err_msg=f"{name} v{v}")
        np.testing.assert_array_equal(many[:len(c["eps"])], c["labels"])
