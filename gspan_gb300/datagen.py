"""Seeded synthetic labelled graphs for the mining workloads.

Every random number comes from a counter-based generator (splitmix64 over
``(seed, stream, index)``) evaluated with numpy integer arithmetic, so a graph
depends only on its parameters and seed and is bit-identical on x86 and Arm
hosts and across numpy versions.

Graphs are returned as the reference's CSR layout (``CSRGraph`` in graph.h:51-65
of haozixu/gSpan): ``offsets int32[n+1]``, ``vlabels int32[n]`` and
``edges int32[m_dir, 3]`` rows ``(from, to, label)``, each undirected edge
stored in both directions, each adjacency sorted by ``(to, label)``
(graph.cc:66-112).  ``to_gspan_text`` writes the same graph in the reference's
text format (graph.cc:38-64) so that the reference's ``convert`` produces the
identical binary file.
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np

_U64 = np.uint64
_GOLDEN = _U64(0x9E3779B97F4A7C15)
_M1 = _U64(0xBF58476D1CE4E5B9)
_M2 = _U64(0x94D049BB133111EB)


def _mix(x: np.ndarray) -> np.ndarray:
    x = x + _GOLDEN
    x = (x ^ (x >> _U64(30))) * _M1
    x = (x ^ (x >> _U64(27))) * _M2
    return x ^ (x >> _U64(31))


def rand_u64(seed: int, stream: int, start: int, count: int) -> np.ndarray:
    """``count`` 64-bit words of stream ``stream`` beginning at ``start``."""
    with np.errstate(over="ignore"):
        key = _mix(np.array([(seed * 0x100000001B3 + stream) & 0xFFFFFFFFFFFFFFFF], dtype=_U64))[0]
        idx = np.arange(start, start + count, dtype=_U64)
        return _mix(idx ^ key)


def rand_unit(seed: int, stream: int, start: int, count: int) -> np.ndarray:
    """Uniform doubles in [0, 1)."""
    return (rand_u64(seed, stream, start, count) >> _U64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)


@dataclass
class CSR:
    offsets: np.ndarray  # int32[n+1]
    vlabels: np.ndarray  # int32[n]
    edges: np.ndarray    # int32[m, 3] (from, to, label)

    @property
    def n(self) -> int:
        return int(self.vlabels.shape[0])

    @property
    def m(self) -> int:
        return int(self.edges.shape[0])

    def to_bytes(self) -> bytes:
        """The reference's binary CSR file (graph.cc:202-214): native-endian int32."""
        head = np.array([self.n, self.m], dtype=np.int32)
        return (head.tobytes() + self.offsets.astype(np.int32).tobytes()
                + self.vlabels.astype(np.int32).tobytes() + self.edges.astype(np.int32).tobytes())

    def save(self, path: str) -> None:
        with open(path, "wb") as f:
            f.write(self.to_bytes())


def load_bin(path: str) -> CSR:
    """Read the reference's binary CSR file (graph.cc:178-200)."""
    raw = np.fromfile(path, dtype=np.int32)
    if raw.size < 2:
        raise ValueError("truncated graph file")
    n, m = int(raw[0]), int(raw[1])
    need = 2 + (n + 1) + n + 3 * m
    if n < 0 or m < 0 or raw.size < need:
        raise ValueError("truncated graph file")
    off = raw[2:2 + n + 1].copy()
    vl = raw[3 + n:3 + 2 * n].copy()
    ed = raw[3 + 2 * n:need].reshape(m, 3).copy()
    return CSR(off, vl, ed)


def csr_from_edge_list(n: int, vlabels: np.ndarray, eu: np.ndarray, ev: np.ndarray,
                       el: np.ndarray) -> CSR:
    """CSR exactly as CSRGraph(Graph&) builds it from ``e u v l`` lines over vertex
    ids 0..n-1: both directions stored, adjacency sorted by (to, label)."""
    eu = np.asarray(eu, dtype=np.int64)
    ev = np.asarray(ev, dtype=np.int64)
    el = np.asarray(el, dtype=np.int64)
    frm = np.concatenate([eu, ev])
    to = np.concatenate([ev, eu])
    lab = np.concatenate([el, el])
    lmin = int(lab.min()) if lab.size else 0
    lbits = max(1, int(lab.max() - lmin).bit_length()) if lab.size else 1
    if frm.size and n > 0 and (2 * math.log2(n) + lbits) < 62:
        # One packed key (from, to, label) sorts in a single pass.
        key = ((frm * n + to) << lbits) | (lab - lmin)
        key.sort()
        lab = (key & ((1 << lbits) - 1)) + lmin
        ft = key >> lbits
        frm, to = ft // n, ft % n
    else:
        order = np.lexsort((lab, to, frm))
        frm, to, lab = frm[order], to[order], lab[order]
    deg = np.bincount(frm, minlength=n) if n else np.zeros(0, dtype=np.int64)
    offsets = np.zeros(n + 1, dtype=np.int64)
    np.cumsum(deg, out=offsets[1:])
    edges = np.stack([frm, to, lab], axis=1).astype(np.int32) if frm.size else np.zeros((0, 3), np.int32)
    return CSR(offsets.astype(np.int32), np.asarray(vlabels, dtype=np.int32), edges)


def to_gspan_text(g: CSR) -> str:
    """gSpan text (``t # 0``, ``v id label``, ``e u v label``) for a CSR whose
    edges are all stored twice; each undirected edge is written once."""
    lines = ["t # 0"]
    lines += [f"v {i} {int(l)}" for i, l in enumerate(g.vlabels)]
    e = g.edges
    if e.shape[0]:
        # one line per undirected edge: keep the from<to copy (self-loops: every
        # second copy, since a self-loop line adds two identical entries)
        fwd = e[e[:, 0] < e[:, 1]]
        loops = e[e[:, 0] == e[:, 1]][::2]
        keep = np.concatenate([fwd, loops]) if loops.size else fwd
        lines += [f"e {int(a)} {int(b)} {int(c)}" for a, b, c in keep]
    return "\n".join(lines) + "\n"


def zipf_labels(n: int, nlabels: int, s: float, seed: int, stream: int = 7) -> np.ndarray:
    """Vertex labels 0..nlabels-1 with p(l) proportional to (l+1)^-s."""
    p = np.arange(1, nlabels + 1, dtype=np.float64) ** (-s)
    cdf = np.cumsum(p / p.sum())
    cdf[-1] = 1.0
    u = rand_unit(seed, stream, 0, n)
    return np.searchsorted(cdf, u, side="right").astype(np.int32)


def _unique_pairs(batches, m: int) -> tuple[np.ndarray, np.ndarray]:
    """First ``m`` distinct unordered pairs (no self-loops) in generation order."""
    us, vs = [], []
    seen = np.zeros(0, dtype=np.int64)
    total = 0
    for a, b in batches:
        lo = np.minimum(a, b)
        hi = np.maximum(a, b)
        ok = lo != hi
        key = lo[ok] * (1 << 32) + hi[ok]
        _, first = np.unique(key, return_index=True)
        first.sort()
        key = key[first]
        fresh = ~np.isin(key, seen)
        key = key[fresh]
        take = key[: m - total]
        seen = np.concatenate([seen, take])
        us.append(take >> 32)
        vs.append(take & 0xFFFFFFFF)
        total += take.size
        if total >= m:
            break
    return np.concatenate(us), np.concatenate(vs)


def erdos_renyi(n: int, m: int, nlabels: int, seed: int, nelabels: int = 1) -> CSR:
    """Simple undirected G(n, m): m distinct pairs drawn uniformly, no self-loops,
    vertex labels uniform over ``nlabels``, edge labels uniform over ``nelabels``."""
    def batches():
        start = 0
        while True:
            cnt = max(1024, int(m * 1.1))
            a = (rand_u64(seed, 1, start, cnt) % _U64(n)).astype(np.int64)
            b = (rand_u64(seed, 2, start, cnt) % _U64(n)).astype(np.int64)
            start += cnt
            yield a, b
    eu, ev = _unique_pairs(batches(), m)
    vl = (rand_u64(seed, 3, 0, n) % _U64(nlabels)).astype(np.int32)
    el = (rand_u64(seed, 4, 0, m) % _U64(nelabels)).astype(np.int32)
    return csr_from_edge_list(n, vl, eu, ev, el)


def chung_lu_weights(n: int, m: int, gamma: float, max_deg: float | None) -> np.ndarray:
    """Expected degrees w_i proportional to (i+1)^(-1/(gamma-1)), summing to 2m,
    capped at ``max_deg`` (the excess is spread over the uncapped vertices)."""
    w = np.arange(1, n + 1, dtype=np.float64) ** (-1.0 / (gamma - 1.0))
    w *= 2.0 * m / w.sum()
    if max_deg is not None:
        for _ in range(64):
            over = w > max_deg
            if not over.any():
                break
            w[over] = max_deg
            free = ~over
            w[free] *= (2.0 * m - max_deg * over.sum()) / w[free].sum()
    return w


def chung_lu(n: int, m: int, gamma: float, nlabels: int, zipf_s: float, seed: int,
             max_deg: float | None = None, nelabels: int = 1) -> CSR:
    """Simple undirected Chung-Lu power-law graph with m distinct edges.  Both
    endpoints of a candidate edge are drawn with probability proportional to the
    weights; self-loops and repeats are redrawn.  Vertex ids are a seeded
    permutation of the weight order, so degree does not follow id."""
    w = chung_lu_weights(n, m, gamma, max_deg)
    cdf = np.cumsum(w / w.sum())
    cdf[-1] = 1.0
    perm = np.argsort(rand_u64(seed, 9, 0, n), kind="stable").astype(np.int64)

    def batches():
        start = 0
        while True:
            cnt = max(4096, int(m * 1.2))
            a = np.searchsorted(cdf, rand_unit(seed, 1, start, cnt), side="right")
            b = np.searchsorted(cdf, rand_unit(seed, 2, start, cnt), side="right")
            start += cnt
            yield perm[np.minimum(a, n - 1)], perm[np.minimum(b, n - 1)]
    eu, ev = _unique_pairs(batches(), m)
    vl = zipf_labels(n, nlabels, zipf_s, seed)
    el = (rand_u64(seed, 4, 0, m) % _U64(nelabels)).astype(np.int32)
    return csr_from_edge_list(n, vl, eu, ev, el)


def random_multigraph(n: int, m: int, nlabels: int, nelabels: int, seed: int,
                      self_loops: bool = True) -> CSR:
    """Small graph with parallel edges (same and different labels) and, if asked,
    self-loops: the corner cases the reference's loader accepts."""
    a = (rand_u64(seed, 11, 0, m) % _U64(max(n, 1))).astype(np.int64)
    b = (rand_u64(seed, 12, 0, m) % _U64(max(n, 1))).astype(np.int64)
    if not self_loops:
        b = np.where(a == b, (b + 1) % max(n, 1), b)
    vl = (rand_u64(seed, 13, 0, n) % _U64(nlabels)).astype(np.int32)
    el = (rand_u64(seed, 14, 0, m) % _U64(nelabels)).astype(np.int32)
    return csr_from_edge_list(n, vl, a, b, el)


# The workloads, by what they are.
def er_3300(seed: int = 0) -> CSR:
    """Erdos-Renyi, 3,300 vertices, 4,700 edges, 6 uniform vertex labels, 1 edge label."""
    return erdos_renyi(3300, 4700, 6, seed)


CL_100K_MAX_DEG = 1400.0


def chung_lu_100k(seed: int = 1) -> CSR:
    """Chung-Lu, 100,000 vertices, 1,080,000 edges, exponent 2.1, expected-degree
    cap 1,400, 29 vertex labels Zipf(1.0), 1 edge label."""
    return chung_lu(100_000, 1_080_000, 2.1, 29, 1.0, seed, max_deg=CL_100K_MAX_DEG)


def chung_lu_3_7m(seed: int = 3) -> CSR:
    """Chung-Lu, 3,700,000 vertices, 16,500,000 edges, exponent 2.3, degree cap
    sqrt(2m), 37 vertex labels Zipf(0.8), 1 edge label."""
    m = 16_500_000
    return chung_lu(3_700_000, m, 2.3, 37, 0.8, seed, max_deg=math.sqrt(2 * m))


def batch_instances(seed: int = 2, count: int = 256) -> tuple[list[CSR], list[int]]:
    """Independent mining instances: Chung-Lu graphs with n log-uniform in
    [1,000, 200,000], average degree uniform in [4, 24], 8 to 32 vertex labels
    Zipf(1.0), exponent 2.1, degree cap sqrt(2m), 1 edge label.  Returns the
    graphs and their min supports (2 % of n)."""
    u = rand_unit(seed, 21, 0, count * 3).reshape(count, 3)
    graphs, sups = [], []
    lo, hi = math.log(1000.0), math.log(200000.0)
    for i in range(count):
        n = int(round(math.exp(lo + u[i, 0] * (hi - lo))))
        m = int(round(n * (4.0 + 20.0 * u[i, 1]) / 2.0))
        nlabels = 8 + min(24, int(u[i, 2] * 25))
        graphs.append(chung_lu(n, m, 2.1, nlabels, 1.0, seed * 1000003 + i, max_deg=math.sqrt(2.0 * m)))
        sups.append(int(0.02 * n))
    return graphs, sups


# Serving: a resident pool of graphs of the three single-graph sizes, and a
# Poisson stream of jobs drawn over it.
SERVING_CLASSES = ("er_3300", "chung_lu_100k", "chung_lu_3_7m")
SERVING_MIX = (0.70, 0.25, 0.05)


def serving_pool(seed: int = 4, per_class: tuple[int, int, int] = (8, 3, 1)) -> list[tuple[int, CSR]]:
    """(size class, graph) pairs with fresh seeds: per_class[c] graphs of
    class c (Erdos-Renyi 3,300 V; Chung-Lu 100,000 V; Chung-Lu 3,700,000 V)."""
    makers = (er_3300, chung_lu_100k, chung_lu_3_7m)
    pool = []
    for c, (make, cnt) in enumerate(zip(makers, per_class)):
        for i in range(cnt):
            pool.append((c, make(seed * 1000 + 100 * c + i)))
    return pool


def serving_jobs(pool_classes: list[int], pool_sizes: list[int], count: int, rate: float = 50.0,
                 seed: int = 4) -> list[tuple[float, int, int, int]]:
    """`count` jobs (arrival seconds, pool index, k, min support): exponential
    inter-arrival times of mean 1/rate, size class drawn by SERVING_MIX, a
    graph of that class uniformly, min support uniform in [1 %, 5 %] of its
    vertex count.  k is 3 or 4 (even odds) for the 3,300-vertex class and 3
    for the others, whose four-edge levels need a level-3 embedding table
    larger than the device at these supports."""
    u = rand_unit(seed, 31, 0, count * 5).reshape(count, 5)
    by_class = [[i for i, c in enumerate(pool_classes) if c == cls] for cls in range(len(SERVING_MIX))]
    cum = np.cumsum(SERVING_MIX)
    t = 0.0
    jobs = []
    for j in range(count):
        t += -math.log(1.0 - u[j, 0]) / rate
        cls = int(np.searchsorted(cum, u[j, 1] * cum[-1], side="right"))
        cls = min(cls, len(SERVING_MIX) - 1)
        members = by_class[cls]
        gi = members[min(len(members) - 1, int(u[j, 2] * len(members)))]
        k = (3 if u[j, 3] < 0.5 else 4) if cls == 0 else 3
        sup = max(1, int(pool_sizes[gi] * (0.01 + 0.04 * u[j, 4])))
        jobs.append((t, gi, k, sup))
    return jobs
