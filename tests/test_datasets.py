"""CPU: synthetic generators are deterministic; bit packing matches the kernel's layout."""
import hashlib

import numpy as np

from vecsearch_gb300 import datasets as D


def test_portable_is_pinned():
    # The golden fixtures depend on these exact bits on every platform.
    x = D.portable(7, 5, 3)
    assert hashlib.sha256(x.tobytes()).hexdigest()[:16] == PORTABLE_HASH
    assert abs(float(D.portable(20000, 8, 1).std()) - 1.0) < 0.02


def test_portable_prefix_property():
    np.testing.assert_array_equal(D.portable(5, 37, 2), D.portable(300, 37, 2)[:5])


def test_pack_bits_layout():
    m = np.zeros(70, bool)
    m[[0, 31, 32, 69]] = True
    w = D.pack_bits(m)
    assert w.dtype == np.uint32 and w.shape == (3,)
    assert w[0] == (1 | (1 << 31)) and w[1] == 1 and w[2] == (1 << 5)
    w2 = D.pack_bits(np.stack([m, ~m]))
    assert w2.shape == (2, 3) and w2[1, 0] == (~w[0] & 0xFFFFFFFF)


def test_clustered_shapes_and_norms():
    x, labels = D.clustered(1000, 16, 8, seed=0)
    assert x.shape == (1000, 16) and labels.max() < 8
    assert np.allclose(np.linalg.norm(x, axis=1), 1.0, atol=1e-5)
    g = D.zipf_groups(5000, 2000)
    assert g.min() >= 0 and g.max() < 2000 and np.bincount(g)[0] > np.bincount(g)[100]


PORTABLE_HASH = "d047114d1bf379c1"  # sha256 prefix of portable(7, 5, 3), fixed when the fixtures were made
