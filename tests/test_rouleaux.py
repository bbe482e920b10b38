"""Rouleau labelling from contact pairs (gc_rouleaux_from_pairs, host code)
against a breadth-first search written here: random graphs, empty input,
self-pairs, repeated pairs, and the error for an index outside the cells."""
import numpy as np
import pytest

from gpucell_gb300 import rouleaux


def _bfs_labels(ncell, pairs):
    adj = [[] for _ in range(ncell)]
    for a, b in pairs:
        adj[a].append(b)
        adj[b].append(a)
    label = [-1] * ncell
    sizes = []
    for c in range(ncell):
        if label[c] >= 0:
            continue
        k = len(sizes)
        label[c] = k
        todo, n = [c], 0
        while todo:
            u = todo.pop()
            n += 1
            for v in adj[u]:
                if label[v] < 0:
                    label[v] = k
                    todo.append(v)
        sizes.append(n)
    return np.array(label, np.int32), np.array(sizes, np.int32)


@pytest.mark.parametrize("seed", range(8))
def test_labels_match_a_breadth_first_search(seed):
    rng = np.random.default_rng(seed)
    ncell = int(rng.integers(1, 300))
    npairs = int(rng.integers(0, 2 * ncell))
    pairs = rng.integers(0, ncell, size=(npairs, 2))
    label, size = rouleaux.from_pairs(ncell, pairs)
    want_label, want_size = _bfs_labels(ncell, pairs.tolist())
    assert np.array_equal(label, want_label)
    assert np.array_equal(size, want_size)
    assert size.sum() == ncell


def test_edge_cases():
    label, size = rouleaux.from_pairs(0, [])
    assert label.size == 0 and size.size == 0
    label, size = rouleaux.from_pairs(4, [])
    assert label.tolist() == [0, 1, 2, 3] and size.tolist() == [1, 1, 1, 1]
    label, size = rouleaux.from_pairs(5, [(3, 3), (4, 2), (2, 4), (4, 2)])
    assert label.tolist() == [0, 1, 2, 3, 2] and size.tolist() == [1, 1, 2, 1]
    label, size = rouleaux.from_pairs(3, [(2, 1), (1, 0)])
    assert label.tolist() == [0, 0, 0] and size.tolist() == [3]
    with pytest.raises(RuntimeError):
        rouleaux.from_pairs(3, [(0, 3)])
    with pytest.raises(RuntimeError):
        rouleaux.from_pairs(3, [(-1, 0)])
