"""Seeded synthetic expression matrices (GEMs) for the Similarity workloads.

KINC's Similarity benchmarks are not tied to a public dataset, so every
workload here is generated: float32 [genes][samples], row-major, NaN for a
missing value, seed ``20260101 + workload``.  Pairs of co-regulated genes are
planted as *modules*: a set of genes that share a per-sample latent mixture
component, so every pair inside a module is a 2-D Gaussian mixture.

Workloads (sizes as named; ``scale`` shrinks genes/samples for small tests):

1. ``pearson``      1,000 x 200;   gene mean ~U(4,12), x ~ N(mean, 2), 5% NaN.
2. ``gmm_spearman`` 5,000 x 1,000; N(8,2), 10% NaN, 10 modules of 500 genes with
                    2-3 components (weights ~Dirichlet(1), correlations
                    ~U(-0.95,0.95), mean offsets ~U(-3,3)).
3. ``dense``        20,000 x 2,000; 8 + L F + e with 50 latent factors, per-gene
                    NaN rate ~U(0, 0.2).
4. ``kmeans``       10,000 x 4,000; N(8,2), per-gene NaN rate ~U(0,0.6), 10
                    modules of 707 genes with 2 components.
5. ``streamed``     30,000 x 500;  N(8,2), 8% NaN, 10 modules of 2,121 genes with
                    2-4 components.
"""
import numpy as np

WORKLOADS = {
    1: dict(name="pearson", genes=1000, samples=200),
    2: dict(name="gmm_spearman", genes=5000, samples=1000),
    3: dict(name="dense", genes=20000, samples=2000),
    4: dict(name="kmeans", genes=10000, samples=4000),
    5: dict(name="streamed", genes=30000, samples=500),
}


def _plant_modules(rng, gem, n_modules, module_genes, comp_range):
    G, S = gem.shape
    module_genes = min(module_genes, G // max(n_modules, 1))
    genes = rng.permutation(G)
    for m in range(n_modules):
        members = genes[m * module_genes:(m + 1) * module_genes]
        if len(members) < 2:
            continue
        c = int(rng.integers(comp_range[0], comp_range[1] + 1))
        w = rng.dirichlet(np.ones(c))
        z = rng.choice(c, size=S, p=w)                      # latent component per sample
        rho = rng.uniform(-0.95, 0.95, size=c)
        u = rng.standard_normal((S, c)).astype(np.float64)  # shared factor per component
        sgn = rng.choice([-1.0, 1.0], size=(len(members), c))
        off = rng.uniform(-3.0, 3.0, size=(len(members), c))
        eps = rng.standard_normal((len(members), S))
        a = np.sqrt(np.abs(rho))[z]                          # [S]
        b = np.sqrt(1.0 - np.abs(rho))[z]
        shared = u[np.arange(S), z]                           # [S]
        vals = 8.0 + off[:, z] + 2.0 * (a[None, :] * sgn[:, z] * shared[None, :] + b[None, :] * eps)
        gem[members, :] = vals.astype(np.float32)


def generate(workload, scale=1.0, genes=None, samples=None, seed=None):
    """Return a float32 [genes][samples] GEM for workload 1..5."""
    spec = WORKLOADS[workload]
    G = genes if genes is not None else max(2, int(round(spec["genes"] * scale)))
    S = samples if samples is not None else max(1, int(round(spec["samples"] * scale)))
    rng = np.random.default_rng(20260101 + workload if seed is None else seed)
    if workload == 1:
        mu = rng.uniform(4.0, 12.0, size=(G, 1))
        gem = (mu + 2.0 * rng.standard_normal((G, S))).astype(np.float32)
        gem[rng.random((G, S)) < 0.05] = np.nan
    elif workload == 2:
        gem = (8.0 + 2.0 * rng.standard_normal((G, S))).astype(np.float32)
        _plant_modules(rng, gem, 10, int(round(500 * G / spec["genes"])) if genes is None else max(2, G // 10),
                       (2, 3))
        gem[rng.random((G, S)) < 0.10] = np.nan
    elif workload == 3:
        k = 50
        L = rng.standard_normal((G, k)).astype(np.float32)
        F = rng.standard_normal((k, S)).astype(np.float32)
        gem = (8.0 + L @ F + 0.5 * rng.standard_normal((G, S))).astype(np.float32)
        rate = rng.uniform(0.0, 0.2, size=(G, 1))
        gem[rng.random((G, S)) < rate] = np.nan
    elif workload == 4:
        gem = (8.0 + 2.0 * rng.standard_normal((G, S))).astype(np.float32)
        _plant_modules(rng, gem, 10, int(round(707 * G / spec["genes"])) if genes is None else max(2, G // 20),
                       (2, 2))
        rate = rng.uniform(0.0, 0.6, size=(G, 1))
        gem[rng.random((G, S)) < rate] = np.nan
    elif workload == 5:
        gem = (8.0 + 2.0 * rng.standard_normal((G, S))).astype(np.float32)
        _plant_modules(rng, gem, 10, int(round(2121 * G / spec["genes"])) if genes is None else max(2, G // 14),
                       (2, 4))
        gem[rng.random((G, S)) < 0.08] = np.nan
    else:
        raise ValueError(f"unknown workload {workload}")
    return np.ascontiguousarray(gem, dtype=np.float32)


def clique_network(blocks, size, seed=20260106, eps=0.002, mid_grid=0.01):
    """A correlation network of `blocks` cliques of `size` genes for the RMT analytic: every pair of a
    clique correlates at the clique's level (a value half-way between two points of a 0.01 threshold
    grid, 0.985 down to 0.695) plus uniform noise of +-eps, so a threshold of that grid keeps or drops
    whole cliques and the pruned matrices stay positive definite.  Returns (genes, x, y, c, r) CMX
    items in pair order (x > y), one cluster per pair."""
    rng = np.random.default_rng(seed)
    levels = 0.985 - mid_grid * rng.integers(0, 30, blocks)
    xs, ys, rs = [], [], []
    for b in range(blocks):
        base = b * size
        for a in range(1, size):
            for c in range(a):
                xs.append(base + a)
                ys.append(base + c)
                rs.append(levels[b] + rng.uniform(-eps, eps))
    xs, ys = np.array(xs, np.int32), np.array(ys, np.int32)
    order = np.lexsort((ys, xs))
    return (blocks * size, xs[order], ys[order], np.zeros(len(xs), np.int8),
            np.array(rs, np.float32)[order])
