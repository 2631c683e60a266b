"""Host-side plan construction (sp_ogs_setup_csr, sp_mesh_box_hex_ids) against the
oracle's restatement of the reference's setup (CPU only)."""
import ctypes

import numpy as np
import pytest

from streamparanumal_gb300 import capi


def product_setup(ids, kind=capi.SIGNED, unique=True):
    N = ids.size
    rsT = np.zeros(N + 1, np.int32)
    ciT = np.zeros(max(N, 1), np.int32)
    rsN = np.zeros(N + 1, np.int32)
    ciN = np.zeros(max(N, 1), np.int32)
    nT, nN = ctypes.c_int32(), ctypes.c_int32()
    capi.call("sp_ogs_setup_csr", N, capi.i64p(ids), kind, int(unique), ctypes.byref(nT),
              capi.i32p(rsT), capi.i32p(ciT), ctypes.byref(nN), capi.i32p(rsN), capi.i32p(ciN))
    rsT = rsT[: nT.value + 1]
    rsN = rsN[: nN.value + 1]
    return dict(rsT=rsT, ciT=ciT[: rsT[-1]], rsN=rsN, ciN=ciN[: rsN[-1]])


def product_ids(nx, ny, nz, p, seed=0):
    ids = np.empty(nx * ny * nz * (p + 1) ** 3, np.int64)
    capi.call("sp_mesh_box_hex_ids", nx, ny, nz, p, seed, capi.i64p(ids))
    return ids


BOXES = [(1, 1, 1, 1), (2, 1, 1, 1), (2, 2, 2, 1), (3, 2, 2, 2), (2, 3, 4, 3), (4, 4, 4, 2),
         (3, 3, 3, 7), (5, 2, 3, 4)]


@pytest.mark.parametrize("box", BOXES)
@pytest.mark.parametrize("seed", [0, 12345])
def test_box_ids_match_reference_min_propagation(lib, orc, box, seed):
    a = product_ids(*box, seed=seed)
    b = orc.box_hex_ids(*box, perm_seed=seed)
    np.testing.assert_array_equal(a, b)


@pytest.mark.parametrize("box", BOXES)
def test_box_global_node_count(lib, box):
    nx, ny, nz, p = box
    ids = product_ids(*box)
    assert np.unique(ids).size == (nx * p + 1) * (ny * p + 1) * (nz * p + 1)


@pytest.mark.parametrize("box", BOXES)
@pytest.mark.parametrize("seed", [0, 7])
def test_setup_matches_oracle_on_boxes(lib, orc, box, seed):
    ids0 = product_ids(*box, seed=seed)
    ids_a, ids_b = ids0.copy(), ids0.copy()
    a = product_setup(ids_a, capi.SIGNED, True)
    b = orc.ogs_setup(ids_b, kind=1, unique=True)
    for key in ("rsT", "ciT", "rsN", "ciN"):
        np.testing.assert_array_equal(a[key], b[key], err_msg=key)
    np.testing.assert_array_equal(ids_a, ids_b)
    # one positive member per group after unique flagging
    assert np.all(np.diff(a["rsN"]) == 1)


def test_box_multiplicities(lib):
    nx, ny, nz, p = 3, 4, 5, 3
    s = product_setup(product_ids(nx, ny, nz, p))
    mult = np.diff(s["rsT"])
    counts = {m: int((mult == m).sum()) for m in (1, 2, 4, 8)}
    assert counts[8] == (nx - 1) * (ny - 1) * (nz - 1)
    assert sum(counts.values()) == mult.size
    assert set(np.unique(mult)) <= {1, 2, 4, 8}
    # rows in order of first appearance, columns ascending
    firsts = s["ciT"][s["rsT"][:-1]]
    assert np.all(np.diff(firsts) > 0)
    for r in range(0, mult.size, 97):
        seg = s["ciT"][s["rsT"][r]:s["rsT"][r + 1]]
        assert np.all(np.diff(seg) > 0)


def random_ids(rng, n, nkeys, zero_frac=0.1, neg_frac=0.3, sparse=False):
    keys = rng.integers(1, nkeys + 1, size=n).astype(np.int64)
    if sparse:
        keys = keys * 1_000_000_007  # forces the sort path of the grouping
    keys[rng.random(n) < neg_frac] *= -1
    keys[rng.random(n) < zero_frac] = 0
    return keys


@pytest.mark.parametrize("kind,unique", [(capi.SIGNED, True), (capi.SIGNED, False),
                                         (capi.UNSIGNED, False), (capi.HALO, False)])
@pytest.mark.parametrize("sparse", [False, True])
@pytest.mark.parametrize("n,nkeys", [(0, 1), (1, 1), (17, 3), (1000, 50), (5000, 4000)])
def test_setup_matches_oracle_on_random_ids(lib, orc, kind, unique, sparse, n, nkeys):
    rng = np.random.default_rng(n * 31 + nkeys + 7 * kind + int(unique) + 3 * int(sparse))
    ids0 = random_ids(rng, n, nkeys, sparse=sparse)
    ids_a, ids_b = ids0.copy(), ids0.copy()
    a = product_setup(ids_a, kind, unique)
    b = orc.ogs_setup(ids_b, kind=kind, unique=unique)
    for key in ("rsT", "ciT", "rsN", "ciN"):
        np.testing.assert_array_equal(a[key], b[key], err_msg=key)
    np.testing.assert_array_equal(ids_a, ids_b)


def test_all_zero_ids_give_an_empty_plan(lib):
    s = product_setup(np.zeros(10, np.int64))
    assert s["rsT"].tolist() == [0] and s["ciT"].size == 0


def test_cfg1_sizes(lib):
    """16x16x16 elements at p=7: 2,097,152 local nodes, 113^3 gathered nodes."""
    ids = product_ids(16, 16, 16, 7)
    s = product_setup(ids)
    assert ids.size == 2_097_152
    assert s["rsT"].size - 1 == 113 ** 3 == 1_442_897
    # the reference's BS8 byte count (BS/BS8/src/bs8Run.cpp:53-61)
    Ng, Nt = 1_442_897, 2_097_152
    assert (Ng + 1) * 4 + Nt * 4 + 2 * Nt * 8 == 47_714_632
