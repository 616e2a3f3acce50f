"""Block partition for a hierarchical (H-matrix) representation of the
collocation matrix (`bem_hmat_partition`, host only; no reference
counterpart).  Checked properties: the blocks tile the (N + M) x N index
space exactly once, admissible blocks meet min(diam) <= eta * dist of their
clusters' bounding boxes, dense blocks pair two leaves, the partition is
deterministic, its dense part shrinks as the mesh is refined, and the
admissible blocks of the oracle's FP64 matrix (icosphere s4, ka = 10) have
low numerical rank."""
import ctypes

import numpy as np
import pytest

from helpers import icosphere


def _rows_cols(subdiv, chief=8, seed=1):
    p, el = icosphere(subdiv)
    c = np.random.default_rng(seed).uniform(-0.3, 0.3, (chief, 3))
    return np.vstack([p, c]), p, el


def _box(x):
    return x.min(axis=0), x.max(axis=0)


def _diam(lo, hi):
    return float(np.linalg.norm(hi - lo))


def _dist(a, b):
    gap = np.maximum(0.0, np.maximum(b[0] - a[1], a[0] - b[1]))
    return float(np.linalg.norm(gap))


def test_partition_tiles_matrix_once(bemlib):
    rows, cols, _ = _rows_cols(4)
    R, N = rows.shape[0], cols.shape[0]
    rp, cp, b = bemlib.hmat_partition(rows, cols, 64, 1.0)
    assert np.array_equal(np.sort(rp), np.arange(R))
    assert np.array_equal(np.sort(cp), np.arange(N))
    cover = np.zeros((R, N), dtype=np.int32)
    for r0, rc, c0, cc, _ in b:
        assert rc > 0 and cc > 0
        cover[r0:r0 + rc, c0:c0 + cc] += 1
    assert (cover == 1).all()
    assert set(np.unique(b[:, 4])) <= {0, 1}


def test_blocks_meet_admissibility_and_leaf_size(bemlib):
    rows, cols, _ = _rows_cols(4)
    leaf, eta = 64, 1.0
    rp, cp, b = bemlib.hmat_partition(rows, cols, leaf, eta)
    xr, xc = rows[rp], cols[cp]
    n_adm = 0
    for r0, rc, c0, cc, adm in b:
        br, bc = _box(xr[r0:r0 + rc]), _box(xc[c0:c0 + cc])
        if adm:
            n_adm += 1
            d = _dist(br, bc)
            assert d > 0.0
            assert min(_diam(*br), _diam(*bc)) <= eta * d * (1 + 1e-12)
        else:
            assert rc <= leaf and cc <= leaf
    assert n_adm > 0


def test_partition_is_deterministic_and_dense_part_shrinks(bemlib):
    frac = []
    for s in (4, 5, 6):
        rows, cols, _ = _rows_cols(s, chief=32)
        out1 = bemlib.hmat_partition(rows, cols, 128, 1.0)
        out2 = bemlib.hmat_partition(rows, cols, 128, 1.0)
        for x, y in zip(out1, out2):
            assert np.array_equal(x, y)
        b = out1[2].astype(np.int64)
        dense = b[b[:, 4] == 0]
        frac.append((dense[:, 1] * dense[:, 3]).sum() / (rows.shape[0] * cols.shape[0]))
    # quarter-ish per refinement once the tree has admissible levels
    assert frac[0] > frac[1] > frac[2]
    assert frac[1] < 0.25 and frac[2] < 0.06, frac


def test_coincident_points_stay_one_cluster(bemlib):
    pts = np.tile([[0.5, -0.25, 1.0]], (300, 1))
    rp, cp, b = bemlib.hmat_partition(pts, pts, 16, 1.0)
    assert b.tolist() == [[0, 300, 0, 300, 0]]
    assert np.array_equal(rp, np.arange(300)) and np.array_equal(cp, np.arange(300))


def test_partition_argument_errors(bemlib):
    rows, cols, _ = _rows_cols(3)
    for leaf, eta in ((0, 1.0), (16, 0.0), (16, float("nan"))):
        with pytest.raises(bemlib.BemError) as e:
            bemlib.hmat_partition(rows, cols, leaf, eta)
        assert e.value.status == bemlib.ERR_INVALID_ARG
    bad = rows.copy()
    bad[3, 1] = np.inf
    with pytest.raises(bemlib.BemError):
        bemlib.hmat_partition(bad, cols, 16, 1.0)
    # a block array too small: BEM_ERR_TOO_LARGE with the count still reported
    L = bemlib.lib()
    rows = np.ascontiguousarray(rows)
    cols = np.ascontiguousarray(cols)
    n = ctypes.c_int(0)
    blocks = np.zeros((4, 5), dtype=np.int32)
    st = L.bem_hmat_partition(rows.ctypes.data, rows.shape[0], cols.ctypes.data, cols.shape[0], 16, 1.0,
                              None, None, blocks.ctypes.data, 4, ctypes.byref(n))
    assert st == bemlib.ERR_TOO_LARGE and n.value > 4


def test_admissible_blocks_are_low_rank_in_oracle_matrix(bemlib, orc):
    """The oracle's FP64 A (icosphere s4, 2562 nodes, 8 CHIEF rows, ka = 10):
    every admissible block of at least 64 x 64 has numerical rank (singular
    values above 1e-6 of the largest entry) below 0.3 of its smaller side."""
    rows, cols, el = _rows_cols(4)
    N = cols.shape[0]
    A, _ = orc.assemble(rows, el, 10.0, N, [("plane", (0.0, 0.0, 1.0), 1.0)],
                        prm=orc.params(near_eta=1.0, near_depth=2))
    rp, cp, b = bemlib.hmat_partition(rows, cols, 64, 1.0)
    Ap = A[rp][:, cp]
    floor = 1e-6 * np.abs(A).max()
    checked = 0
    for r0, rc, c0, cc, adm in b:
        if not adm or min(rc, cc) < 64:
            continue
        s = np.linalg.svd(Ap[r0:r0 + rc, c0:c0 + cc], compute_uv=False)
        assert (s > floor).sum() < 0.3 * min(rc, cc)
        checked += 1
    assert checked >= 100


def test_system_partition_shares_the_node_tree(bemlib):
    """Rows = nodes in the column tree's order, then the CHIEF points: the
    blocks tile (N + M) x N once, no block mixes node and CHIEF rows, every
    node-row range is a column cluster, and the admissible blocks meet the
    criterion with the renumbered points."""
    _, nodes, _ = _rows_cols(4)
    chief = np.random.default_rng(1).uniform(-0.3, 0.3, (8, 3))
    N, M = nodes.shape[0], chief.shape[0]
    node_perm, chief_perm, b = bemlib.hmat_partition_system(nodes, chief, 64, 1.0)
    assert np.array_equal(np.sort(node_perm), np.arange(N))
    assert np.array_equal(np.sort(chief_perm), np.arange(M))
    cover = np.zeros((N + M, N), dtype=np.int32)
    for r0, rc, c0, cc, _ in b:
        cover[r0:r0 + rc, c0:c0 + cc] += 1
        assert r0 + rc <= N or r0 >= N
    assert (cover == 1).all()
    col_ranges = {(c0, cc) for _, _, c0, cc, _ in b}
    assert {(r0, rc) for r0, rc, _, _, _ in b if r0 < N} <= col_ranges
    # the node tree is the plain partition's column tree
    _, cp, _ = bemlib.hmat_partition(np.vstack([nodes, chief]), nodes, 64, 1.0)
    assert np.array_equal(node_perm, cp)
    xr = np.vstack([nodes[node_perm], chief[chief_perm]])
    xc = nodes[node_perm]
    for r0, rc, c0, cc, adm in b:
        if adm:
            br, bc = _box(xr[r0:r0 + rc]), _box(xc[c0:c0 + cc])
            d = _dist(br, bc)
            assert d > 0.0 and min(_diam(*br), _diam(*bc)) <= d * (1 + 1e-12)
    # without CHIEF points the rows are the nodes alone
    p2, c2, b2 = bemlib.hmat_partition_system(nodes, None, 64, 1.0)
    assert np.array_equal(p2, node_perm) and c2.size == 0
    assert (b2[:, 0] + b2[:, 1]).max() == N
