"""Seeded synthetic systems for the workloads of the range-limited force path.

Positions are generated in FP64 and cast to FP32; seeds are 20191117 + workload id (replica r of
the batched workload adds 1000*r).  Units: Angstrom, kcal/mol, amu, fs, elementary charge.

Workloads (all periodic):
  lj1728      1,728 argon atoms in a 25.5 A cube, rc 8.5 (3x3x3 cells), LJ only.  A 3.0 A minimum
              separation at 0.104 /A^3 is geometrically impossible (hard-sphere packing 1.47), so
              the atoms sit on a 12^3 simple-cubic lattice (2.125 A) with +-0.1 A uniform jitter.
  ljc92k      92,224 atoms in 108.86 x 108.86 x 77.76 A, rc 12 (9x9x6 cells), 4 LJ types
              (sigma 2.0-3.8, eps 0.02-0.2, Lorentz-Berthelot), charges +-0.42 e net neutral,
              uniform placement at 0.1 /A^3 with 1.0 A minimum separation.
  ljc1m       1,048,576 atoms in a 224 A cube, rc 10 (22^3 cells), 16 types, charges U(-0.8, 0.8)
              shifted to net zero; 1.0 A minimum separation as for ljc92k (without one, random
              overlaps give pair forces beyond the int64 fixed-point range).
  batch512    512 independent replicas, N log-uniform in [500, 20000] (sizes drawn from seed
              20191117 + 4), cubic box L = (N / 0.1)^(1/3), rc 10; each replica (seed
              20191117 + 4 + 1000 r) is argon-like (sigma 3.4, epsilon 0.238, 39.95 amu) with
              +-0.42 e net-neutral charges, placed uniformly with a 1.0 A minimum separation.
              Replicas below ~2,700 atoms have fewer than 3 cells per axis, and below ~800 the
              box edge is under 2 rc.
"""
from __future__ import annotations

import dataclasses

import numpy as np

KCAL_PER_AMU_A2_FS2 = 1.0 / 4.184e-4   # (amu A^2/fs^2) -> kcal/mol
KB_KCAL = 0.0019872041                   # kcal/(mol K)
COULOMB_K = 332.0637                     # kcal A / (mol e^2)


@dataclasses.dataclass
class System:
    name: str
    box: tuple
    cutoff: float
    ncell: tuple
    pos: np.ndarray          # (n,3) float32 in [0, box)
    vel: np.ndarray          # (n,3) float32, A/fs
    q: np.ndarray | None     # (n,) float32 or None
    type: np.ndarray         # (n,) int32
    sigma: list
    epsilon: list
    mass: list
    coulomb_k: float
    # first table point r2 = 2^table_min_log2: the square of the workload's minimum separation
    # (rounded down to a power of two), so that pairs pushed closer during MD are evaluated at a
    # finite, representable force instead of the far larger one at the library default 2^-2
    table_min_log2: int = -2

    @property
    def n(self) -> int:
        return self.pos.shape[0]

    def params(self, **kw):
        from . import default_params
        T = len(self.sigma)
        p = default_params(box=self.box, cutoff=self.cutoff, ncell=self.ncell, ntypes=T,
                           sigma=self.sigma, epsilon=self.epsilon, mass=self.mass,
                           coulomb_k=self.coulomb_k, table_min_log2=self.table_min_log2)
        for k, v in kw.items():
            setattr(p, k, v)
        return p


def wrap_into_box(pos: np.ndarray, box) -> np.ndarray:
    """FP32 positions in [0, L) on every axis."""
    out = np.asarray(pos, dtype=np.float32).copy()
    for d in range(3):
        L = np.float32(box[d])
        c = out[:, d]
        c[c >= L] -= L
        c[c < 0] += L
        c[(c >= L) | (c < 0)] = 0.0
    return out


def maxwell(n: int, mass: np.ndarray, temp: float, rng: np.random.Generator) -> np.ndarray:
    """Maxwell velocities (A/fs) at temp with the centre-of-mass velocity removed."""
    sd = np.sqrt(KB_KCAL * temp / mass / KCAL_PER_AMU_A2_FS2)
    v = rng.standard_normal((n, 3)) * sd[:, None]
    v -= (mass[:, None] * v).sum(0) / mass.sum()
    return v.astype(np.float32)


def uniform_min_sep(n: int, box, dmin: float, rng: np.random.Generator) -> np.ndarray:
    """n uniform points in the periodic box with no pair closer than dmin (random sequential
    re-draws of one member of each violating pair)."""
    from scipy.spatial import cKDTree
    box = np.asarray(box, dtype=np.float64)
    pos = rng.random((n, 3)) * box
    for _ in range(200):
        tree = cKDTree(pos, boxsize=box)
        pairs = tree.query_pairs(dmin, output_type="ndarray")
        if len(pairs) == 0:
            return pos
        bad = np.unique(pairs[:, 1])
        pos[bad] = rng.random((len(bad), 3)) * box
    raise RuntimeError("could not place particles with the requested minimum separation")


def lj1728(seed_offset: int = 0) -> System:
    rng = np.random.default_rng(20191117 + 1 + seed_offset)
    L = 25.5
    a = L / 12
    g = (np.arange(12) + 0.5) * a
    X, Y, Z = np.meshgrid(g, g, g, indexing="ij")
    pos = np.stack([X.ravel(), Y.ravel(), Z.ravel()], 1)
    pos += rng.uniform(-0.1, 0.1, pos.shape)
    pos = wrap_into_box(pos, (L, L, L))
    m = np.full(len(pos), 39.95)
    return System("lj1728", (L, L, L), 8.5, (3, 3, 3), pos, maxwell(len(pos), m, 300.0, rng),
                  None, np.zeros(len(pos), np.int32), [3.4], [0.238], [39.95], 0.0, table_min_log2=0)


def ljc92k(n: int = 92224, box=(108.86, 108.86, 77.76), seed_offset: int = 0) -> System:
    rng = np.random.default_rng(20191117 + 2 + seed_offset)
    pos = wrap_into_box(uniform_min_sep(n, box, 1.0, rng), box)
    sigma = [2.0, 2.6, 3.2, 3.8]
    eps = [0.02, 0.08, 0.14, 0.20]
    mass = [12.011, 14.007, 15.999, 39.95]
    t = rng.integers(0, 4, n).astype(np.int32)
    q = np.full(n, 0.42)
    q[: n // 2] = -0.42
    rng.shuffle(q)
    m = np.asarray(mass)[t]
    ncell = tuple(int(np.floor(np.float32(b) / np.float32(12.0))) for b in box)
    return System("ljc92k", tuple(box), 12.0, ncell, pos, maxwell(n, m, 300.0, rng),
                  q.astype(np.float32), t, sigma, eps, mass, COULOMB_K, table_min_log2=0)


def ljc1m(n: int = 1048576, L: float = 224.0, seed_offset: int = 0) -> System:
    rng = np.random.default_rng(20191117 + 5 + seed_offset)
    pos = wrap_into_box(uniform_min_sep(n, (L, L, L), 1.0, rng), (L, L, L))
    T = 16
    sigma = list(rng.uniform(2.5, 3.8, T))
    eps = list(rng.uniform(0.05, 0.25, T))
    mass = list(rng.uniform(12.0, 40.0, T))
    t = rng.integers(0, T, n).astype(np.int32)
    q = rng.uniform(-0.8, 0.8, n)
    q -= q.mean()
    m = np.asarray(mass)[t]
    nc = int(np.floor(np.float32(L) / np.float32(10.0)))
    return System("ljc1m", (L, L, L), 10.0, (nc, nc, nc), pos, maxwell(n, m, 300.0, rng),
                  q.astype(np.float32), t, sigma, eps, mass, COULOMB_K, table_min_log2=0)


def small_ljc(n: int, L: float, cutoff: float, seed: int, ntypes: int = 4,
              dmin: float = 1.0) -> System:
    """A small LJ+Coulomb system of the ljc92k kind (for parity tests)."""
    rng = np.random.default_rng(seed)
    box = (L, L, L)
    pos = wrap_into_box(uniform_min_sep(n, box, dmin, rng), box)
    sigma = [2.0, 2.6, 3.2, 3.8][:ntypes]
    eps = [0.02, 0.08, 0.14, 0.20][:ntypes]
    mass = [12.011, 14.007, 15.999, 39.95][:ntypes]
    t = rng.integers(0, ntypes, n).astype(np.int32)
    q = np.where(rng.random(n) < 0.5, -0.42, 0.42)
    m = np.asarray(mass)[t]
    nc = int(np.floor(np.float32(L) / np.float32(cutoff)))
    return System("small_ljc", box, cutoff, (nc, nc, nc), pos, maxwell(n, m, 300.0, rng),
                  q.astype(np.float32), t, sigma, eps, mass, COULOMB_K,
                  table_min_log2=int(np.floor(np.log2(dmin * dmin))) if dmin > 0 else -2)


def replica(n: int, r: int, density: float = 0.1, cutoff: float = 10.0, dmin: float = 1.0) -> System:
    """Replica r of the batched workload: n argon-like atoms with +-0.42 e charges in a cube
    at `density`."""
    rng = np.random.default_rng(20191117 + 4 + 1000 * r)
    L = float((n / density) ** (1.0 / 3.0))
    box = (L, L, L)
    pos = wrap_into_box(uniform_min_sep(n, box, dmin, rng), box)
    q = np.full(n, 0.42)
    q[: n // 2] = -0.42
    if n % 2:
        q[-1] = 0.0
    rng.shuffle(q)
    m = np.full(n, 39.95)
    nc = max(1, int(np.floor(np.float32(L) / np.float32(cutoff))))
    return System(f"replica{r}", box, cutoff, (nc, nc, nc), pos, maxwell(n, m, 300.0, rng),
                  q.astype(np.float32), np.zeros(n, np.int32), [3.4], [0.238], [39.95], COULOMB_K,
                  table_min_log2=int(np.floor(np.log2(dmin * dmin))) if dmin > 0 else -2)


def batch_sizes(count: int = 512, lo: int = 500, hi: int = 20000) -> np.ndarray:
    """Replica sizes of the batched workload: log-uniform in [lo, hi]."""
    rng = np.random.default_rng(20191117 + 4)
    return np.exp(rng.uniform(np.log(lo), np.log(hi), count)).round().astype(np.int64)


def batch512(count: int = 512) -> list:
    return [replica(int(n), r) for r, n in enumerate(batch_sizes(count))]


def concat(reps: list):
    """Concatenated arrays of a replica list: (pos, vel, q, type, [(n, box), ...])."""
    pos = np.concatenate([s.pos for s in reps]).astype(np.float32)
    vel = np.concatenate([s.vel for s in reps]).astype(np.float32)
    q = np.concatenate([s.q for s in reps]).astype(np.float32)
    t = np.concatenate([s.type for s in reps]).astype(np.int32)
    return pos, vel, q, t, [(s.n, s.box) for s in reps]


def _grow_chains(k: int, length: int, L: float, bond: float, th: float, rng) -> np.ndarray:
    """k chains of `length` beads at once: (k, length, 3), bond length `bond`, bond angle th,
    torsions near 60 / 180 / 300 degrees, first beads uniform in the cube [0, L)^3 (unwrapped)."""
    unit = lambda v: v / np.linalg.norm(v, axis=-1, keepdims=True)
    pos = np.zeros((k, length, 3))
    pos[:, 0] = rng.random((k, 3)) * L
    if length > 1:
        pos[:, 1] = pos[:, 0] + bond * unit(rng.standard_normal((k, 3)))
    for s in range(2, length):
        b1 = unit(pos[:, s - 1] - pos[:, s - 2])
        if s == 2:
            u = unit(np.cross(b1, rng.standard_normal((k, 3))))
        else:
            n0 = unit(np.cross(pos[:, s - 2] - pos[:, s - 3], b1))
            phi = np.deg2rad(rng.choice([60.0, 180.0, 300.0], k) + rng.normal(0, 10, k))[:, None]
            u = np.cos(phi) * n0 + np.sin(phi) * np.cross(b1, n0)
        pos[:, s] = pos[:, s - 1] + bond * (np.cos(np.pi - th) * b1 + np.sin(np.pi - th) * u)
    return pos


def chains(nchains: int, length: int, L: float, seed: int, cutoff: float = 10.0, bond: float = 1.53,
           angle_deg: float = 111.0, dmin: float = 1.2, sigma: float = 1.0, epsilon: float = 0.05,
           mass: float = 14.0):
    """Linear chains of `length` beads grown in a periodic cube of edge L (bond `bond` A, bond
    angle `angle_deg`, torsions drawn near 60/180/300 degrees, no two beads closer than dmin;
    dmin <= 0 skips that check, for large timing workloads),
    with harmonic bonds, angles (+ Urey-Bradley on every other angle) and 3-fold plus 1-fold
    dihedral terms.  Returns (System, {"bonds": (atoms, params), "angles": ..., "dihedrals": ...});
    the soft, small-sigma LJ keeps bonded neighbours (which also interact through the pair path)
    well-behaved."""
    from scipy.spatial import cKDTree
    rng = np.random.default_rng(seed)
    th = np.deg2rad(angle_deg)
    pos = []
    if dmin <= 0:
        pos = [np.mod(c, L) for c in _grow_chains(nchains, length, L, bond, th, rng)]
    for _ in range(1000):
        if len(pos) == nchains:
            break
        for cand in _grow_chains(nchains - len(pos), length, L, bond, th, rng):
            cand = np.mod(cand, L)
            allp = np.concatenate(pos + [cand]) if pos else cand
            if len(cKDTree(allp, boxsize=L).query_pairs(dmin)) == 0:
                pos.append(cand)
    if len(pos) < nchains:
        raise RuntimeError("could not place the chains")
    P = wrap_into_box(np.concatenate(pos), (L, L, L))
    n = len(P)
    idx = np.arange(n).reshape(nchains, length)
    b_at = np.stack([idx[:, :-1].ravel(), idx[:, 1:].ravel()], 1)
    b_par = np.tile([300.0, bond], (len(b_at), 1))
    a_at = np.stack([idx[:, :-2].ravel(), idx[:, 1:-1].ravel(), idx[:, 2:].ravel()], 1)
    a_par = np.tile([60.0, th, 0.0, 0.0], (len(a_at), 1))
    a_par[::2, 2] = 20.0
    a_par[::2, 3] = 2.0 * bond * np.sin(th / 2)
    d1 = np.stack([idx[:, :-3].ravel(), idx[:, 1:-2].ravel(), idx[:, 2:-1].ravel(), idx[:, 3:].ravel()], 1)
    d_at = np.concatenate([d1, d1])
    d_par = np.concatenate([np.tile([1.4, 3, 0.0], (len(d1), 1)), np.tile([0.3, 1, np.pi], (len(d1), 1))])
    m = np.full(n, mass)
    cut = min(cutoff, L / 3)
    nc = int(np.floor(np.float32(L) / np.float32(cut)))
    sysm = System("chains", (L, L, L), cut, (nc, nc, nc), P, maxwell(n, m, 300.0, rng), None,
                  np.zeros(n, np.int32), [sigma], [epsilon], [mass], 0.0)
    return sysm, {"bonds": (b_at, b_par), "angles": (a_at, a_par), "dihedrals": (d_at, d_par)}
