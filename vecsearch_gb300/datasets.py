"""Seeded synthetic inputs for the exact k-NN workloads.

* :func:`clustered` - the Gaussian-mixture workload: centroids ~ N(0, 1) in d
  dims, rows = centroid + sigma * N(0, 1), optionally L2-normalised (cosine
  search on unit rows). Fast (numpy ``default_rng``); used by the benchmark.
* :func:`portable` - integer-only generator (splitmix64 counters, a sum of four
  16-bit uniforms scaled to unit variance, exact IEEE float64 steps). Its
  output is bit-identical on every platform and numpy version, so committed
  golden outputs can be regenerated from a seed.
* :func:`zipf_groups` - one integer group label per row, Zipf(s) over G groups.
* :func:`group_masks` - per-query bit masks (uint32 words) selecting one group.
"""
import numpy as np

_GOLDEN = np.uint64(0x9E3779B97F4A7C15)
_M1 = np.uint64(0xBF58476D1CE4E5B9)
_M2 = np.uint64(0x94D049BB133111EB)


def _splitmix64(seed, count):
    with np.errstate(over="ignore"):
        z = (np.arange(1, count + 1, dtype=np.uint64) + np.uint64(seed) * np.uint64(1 << 32)) * _GOLDEN
        z = (z ^ (z >> np.uint64(30))) * _M1
        z = (z ^ (z >> np.uint64(27))) * _M2
        return z ^ (z >> np.uint64(31))


def _normalize_exact(x):
    """Row L2 normalisation with a fixed float64 operation order (platform independent)."""
    x64 = x.astype(np.float64)
    s = x64[:, 0] * x64[:, 0]
    for j in range(1, x64.shape[1]):
        s = s + x64[:, j] * x64[:, j]
    s = np.sqrt(s)
    s[s < 1e-12] = 1e-12
    return (x64 / s[:, None]).astype(np.float32)


def portable(n, d, seed, normalize=False):
    """n x d float32 rows, approximately N(0, 1), identical on every platform."""
    z = _splitmix64(seed, n * d)
    m = np.uint64(0xFFFF)
    s = ((z & m) + ((z >> np.uint64(16)) & m) + ((z >> np.uint64(32)) & m) + (z >> np.uint64(48)))
    x = ((s.astype(np.float64) - 131070.0) / 37837.0).astype(np.float32).reshape(n, d)
    return _normalize_exact(x) if normalize else x


def portable_uniform_u32(seed, count):
    """count uint32 values from the same splitmix64 stream family (portable)."""
    return (_splitmix64(seed, count) >> np.uint64(32)).astype(np.uint32)


def portable_clustered(n, d, n_clusters, sigma=0.35, seed=0, centroid_seed=2, unit=True):
    """Platform-independent Gaussian-mixture rows: centroid[label] + sigma * noise, optionally unit."""
    c = portable(n_clusters, d, centroid_seed)
    labels = (portable_uniform_u32(seed + 7919, n) % np.uint32(n_clusters)).astype(np.int64)
    x = c[labels] + np.float32(sigma) * portable(n, d, seed)
    return (_normalize_exact(x) if unit else x.astype(np.float32)), labels


def portable_mask(n, frac, seed):
    """Bernoulli(frac) row mask as uint8, platform-independent."""
    u = portable_uniform_u32(seed, n).astype(np.float64) / 4294967296.0
    return (u < frac).astype(np.uint8)


def normalize(x):
    """L2-normalise rows so inner product equals cosine similarity (eps 1e-12)."""
    x = np.ascontiguousarray(x, dtype=np.float32)
    return x / np.maximum(np.linalg.norm(x, axis=1, keepdims=True), 1e-12)


def clustered(n, d, n_clusters, sigma=0.35, seed=0, centroid_seed=2, unit=True, chunk=65536):
    """n x d float32 rows from a Gaussian mixture with uniform cluster weights.

    Centroids come from ``centroid_seed`` so that base rows (seed 0) and queries
    (seed 1) share one mixture. Returns (rows, cluster label per row).
    """
    c = np.random.default_rng(centroid_seed).standard_normal((n_clusters, d), dtype=np.float32)
    rng = np.random.default_rng(seed)
    labels = rng.integers(0, n_clusters, n, dtype=np.int64)
    x = np.empty((n, d), np.float32)
    for i in range(0, n, chunk):
        m = min(chunk, n - i)
        block = rng.standard_normal((m, d), dtype=np.float32)
        block *= np.float32(sigma)
        block += c[labels[i:i + m]]
        if unit:
            block /= np.maximum(np.linalg.norm(block, axis=1, keepdims=True), np.float32(1e-12))
        x[i:i + m] = block
    return x, labels


def zipf_groups(n, n_groups=2000, s=1.1, seed=3):
    """Group label per row: P(group g) proportional to 1 / (g + 1)^s, g < n_groups."""
    p = 1.0 / np.arange(1, n_groups + 1, dtype=np.float64) ** s
    p /= p.sum()
    return np.random.default_rng(seed).choice(n_groups, size=n, p=p).astype(np.int32)


def pack_bits(mask):
    """bool/uint8 array [..., n] -> uint32 words [..., ceil(n / 32)], bit i of word w = row 32 w + i."""
    mask = np.asarray(mask) != 0
    n = mask.shape[-1]
    nw = (n + 31) // 32
    pad = nw * 32 - n
    if pad:
        mask = np.concatenate([mask, np.zeros(mask.shape[:-1] + (pad,), bool)], axis=-1)
    b = np.packbits(mask, axis=-1, bitorder="little")
    return np.ascontiguousarray(b).view("<u4").astype(np.uint32, copy=False)


def group_masks(groups, query_groups):
    """Per-query uint32 bit masks: query i may return rows whose group equals query_groups[i]."""
    groups = np.asarray(groups)
    out = np.empty((len(query_groups), (len(groups) + 31) // 32), np.uint32)
    for i, g in enumerate(query_groups):
        out[i] = pack_bits(groups == g)
    return out
