"""Synthetic energy-system model of the replica sampler, and the static move tables.

The reference reads a PyPSA-Eur network from HDF5 (``src/system.jl:35`` ``load_system``); that
data is not available, so this module generates a seeded synthetic network of the same form
(nodes, AC lines, one unit per node and carrier) with the sizes of the benchmark configurations:

* N nodes on a random connected graph (Euclidean minimum spanning tree plus the shortest extra
  edges, L lines in total), susceptance 1, ratings lognormal(log 1 GW, 0.5);
* per node: onshore wind, solar, OCGT (the dispatchable unit, field ``g_OCGT``), battery (6 h)
  and H2 (168 h) storage; offshore wind on ``n_off`` nodes;
* capacities uniform in [0, 20 GW] (box [0, 20 GW]); marginal costs uniform in [0, 80] EUR/MWh;
* demand: node scale lognormal(log 2 GW, 0.6) x (1 + 0.15 sin daily + 0.2 cos seasonal) plus a
  weather anomaly of standard deviation 0.05 of the scale;
* capacity factors: logistic of a 2-regime Markov-switching VAR(1) anomaly with diagonal AR 0.9,
  switch probability 0.02 and N(0, 0.3^2) innovations.

Everything is node-valued (the device state of the reference's GPU port, ``docs/system/device.md``
section 1): the move directions that the reference takes from its sparse graph-Haar bases
(``src/spatial.jl:112`` ``haar_basis``) are built here once as node-space columns ("atoms").

Builder decisions (deviations from the reference's data pipeline, all on the data side):
the Fiedler vector that orders child cells (``src/spatial.jl:183``) is sign-normalised (first
non-zero component negative); the weather prior is defined directly on node anomalies (its
covariances are multiples of the identity, so that is the same law as in any orthonormal basis);
the availability map is the logistic function instead of the clamp of ``src/energy.jl:515``.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

# unit kinds of the flat capacity vector
KIND_REN, KIND_DISP, KIND_STOR = 0, 1, 2
# v-field roles (src/local.jl:36)
ROLE_THETA, ROLE_GEN, ROLE_SE = 1, 3, 6

# the plain local families and their rates (src/local.jl:1912 plain_families), then the compensated
# transport families tpot and tsoc of the flow design (src/flowmoves.jl:333), off in the plain sweep
FAMILIES = ("unit", "pair", "xpair", "xlocc", "xloc", "potential", "cellpair", "cell", "spair", "tpot", "tsoc")
FAMILY_RATES = (0.3, 0.25, 0.03, 0.08, 0.04, 0.1, 0.1, 0.1, 0.3, 0.0, 0.0)

# Langevin offsets kappa_s per carrier (src/replicas.jl:522 LANGEVIN_KAPPA)
LANGEVIN_KAPPA = {"onwind": 500.0, "solar": 1000.0, "offwind": 200.0, "gas": 300.0, "OCGT": 300.0,
                  "battery": 100.0, "H2": 100.0}


@dataclass
class Atoms:
    """Sparse node-space columns of one v field (CSR by atom)."""
    role: int
    ptr: np.ndarray      # int32 [natoms+1]
    idx: np.ndarray      # int32: node (theta) or flat unit (gen, storage)
    val: np.ndarray      # float64


@dataclass
class SynthModel:
    N: int
    L: int
    T: int
    dt: float
    seed: int
    # network
    coords: np.ndarray
    country: np.ndarray          # int32 [N], 0-based
    comp: np.ndarray             # int32 [N], AC component, 0-based
    bus0: np.ndarray
    bus1: np.ndarray
    line_b: np.ndarray
    line_s: np.ndarray
    # capacity units (flat, in k-field order: renewables, dispatchable, storage)
    carriers: list               # carrier name per capacity group
    unit_kind: np.ndarray        # int32 [K]
    unit_group: np.ndarray       # int32 [K] index into carriers
    unit_bus: np.ndarray         # int32 [K]
    unit_mc: np.ndarray
    unit_capex: np.ndarray
    unit_lo: np.ndarray
    unit_hi: np.ndarray
    unit_series: np.ndarray      # weather series of a renewable, -1 otherwise
    unit_avail: np.ndarray       # constant availability of a dispatchable unit
    unit_hours: np.ndarray       # storage energy-to-power ratio
    unit_eta_in: np.ndarray
    unit_eta_out: np.ndarray
    unit_qt: np.ndarray          # storage inflow per unit power
    k0: np.ndarray               # initial capacities (MW)
    # index maps of the sub-populations
    disp: np.ndarray             # flat capacity index of every dispatchable unit (order = g fields)
    stor: np.ndarray             # flat capacity index of every storage unit (order = se fields)
    ren: np.ndarray
    # weather
    n0: int
    series_field: np.ndarray     # 0 load, 1 onwind, 2 offwind, 3 solar
    series_node: np.ndarray
    xbar: np.ndarray             # [n0, T] climatology (physical units)
    wscale: np.ndarray           # [n0] physical scale of the anomaly
    K: int
    Ptr: np.ndarray
    pi0: np.ndarray
    phi: np.ndarray              # [K, n0] diagonal AR coefficient
    mu: np.ndarray               # [K, n0, 3] harmonic regime mean (const, cos, sin)
    sig: np.ndarray              # [K, n0] innovation sd
    sig0: np.ndarray             # [n0] sd of the first step
    # prices and temperatures
    c_shed: float = 3000.0
    c_dump: float = 5.0
    c_viol: float = 3000.0
    gamma_k: float = 10.0
    kappa0: float = 1.0
    beta_v: float = 4e-5
    beta_k: float = 4e-8
    physical: bool = True        # reference measure (configs/device40_replica.toml: measure = "physical")
    # move tables
    atoms: list = field(default_factory=list)    # Atoms per v field: theta, g groups, se groups
    nodelines_ptr: np.ndarray = None
    nodelines: np.ndarray = None
    units_ptr: np.ndarray = None                  # dispatchable units per node (index into disp)
    units_at: np.ndarray = None
    stor_ptr: np.ndarray = None                   # storage units per node (index into stor)
    stor_at: np.ndarray = None
    qcum: np.ndarray = None                       # cell-move level probabilities (cumulative)
    cell_ptr: np.ndarray = None                   # [ncell_total+1] -> units (index into disp)
    cell_units: np.ndarray = None
    cell_level_ptr: np.ndarray = None             # [nlev+1] -> cells
    xpart_ptr: np.ndarray = None                  # xloc partners per node
    xpart: np.ndarray = None
    xnod_ptr: np.ndarray = None                   # per (node, partner) pair -> theta nodes
    xnod: np.ndarray = None
    xval: np.ndarray = None
    xlk_ptr: np.ndarray = None                    # per pair -> leak nodes
    xlkn: np.ndarray = None
    xlkg: np.ndarray = None
    reroute: np.ndarray = None                    # [N, N] grounded Laplacian inverse (column n: e_n response)

    @property
    def Kunits(self):
        return len(self.unit_kind)

    @property
    def D(self):
        return len(self.disp)

    @property
    def S(self):
        return len(self.stor)


# --------------------------------------------------------------------------------------------
# graph-Haar bases (src/spatial.jl:112-221)
# --------------------------------------------------------------------------------------------

def haar_basis(partitions, support, edges=None, drop_top=False, weights=None):
    """Sparse orthonormal graph-Haar basis on ``support`` (``src/spatial.jl:112`` ``haar_basis``).

    Returns the columns as a list of (rows, values) with rows ascending, and the counts per level.
    """
    S = len(support)
    wts = np.ones(S) if weights is None else np.asarray(weights, float)
    pos = {int(n): i for i, n in enumerate(support)}
    labels = []
    prev = [0] * S
    for lab in partitions:
        key = {}
        cur = []
        for i in range(S):
            kk = (prev[i], int(lab[support[i]]))
            if kk not in key:
                key[kk] = len(key) + 1
            cur.append(key[kk])
        labels.append(cur)
        prev = cur
    cols = []

    def addvec(plus, minus):
        if not minus:
            a = 1.0 / math.sqrt(sum(wts[i] ** 2 for i in plus))
            cols.append((list(plus), [a * wts[i] for i in plus]))
            return
        sp = sum(wts[i] ** 2 for i in plus)
        sm = sum(wts[i] ** 2 for i in minus)
        nrm = math.sqrt(1.0 / sp + 1.0 / sm)
        rows = list(plus) + list(minus)
        vals = [wts[i] / sp / nrm for i in plus] + [-wts[i] / sm / nrm for i in minus]
        order = np.argsort(rows, kind="stable")
        cols.append(([rows[o] for o in order], [vals[o] for o in order]))

    counts = []
    if not drop_top:
        for c in range(1, max(labels[0], default=0) + 1):
            addvec([i for i in range(S) if labels[0][i] == c], [])
    counts.append(len(cols))
    W = {}
    if edges is not None:
        for a, b, w in edges:
            if int(a) in pos and int(b) in pos:
                i, j = pos[int(a)], pos[int(b)]
                if i == j:
                    continue
                kk = (min(i, j), max(i, j))
                W[kk] = W.get(kk, 0.0) + float(w)
    for q in range(1, len(labels)):
        par, ch = labels[q - 1], labels[q]
        for p in range(1, max(par, default=0) + 1):
            members = [i for i in range(S) if par[i] == p]
            kids = list(dict.fromkeys(ch[i] for i in members))
            if len(kids) < 2:
                continue
            groups = [[i for i in members if ch[i] == c] for c in kids]
            groups = _order_groups(groups, W)
            _bisect_contrasts(addvec, groups)
        counts.append(len(cols))
    # droptol 1e-14 (src/spatial.jl:34)
    cols = [([r for r, v in zip(rs, vs) if abs(v) > 1e-14], [v for v in vs if abs(v) > 1e-14]) for rs, vs in cols]
    return cols, counts, labels


def _order_groups(groups, W):
    """Order cells along the Fiedler vector of their quotient graph (``src/spatial.jl:183``)."""
    K = len(groups)
    if K <= 2 or not W:
        return groups
    g = {i: k for k, grp in enumerate(groups) for i in grp}
    Lq = np.zeros((K, K))
    for (i, j), w in W.items():
        if i in g and j in g:
            a, b = g[i], g[j]
            if a == b:
                continue
            Lq[a, a] += w
            Lq[b, b] += w
            Lq[a, b] -= w
            Lq[b, a] -= w
    if not Lq.any():
        return groups
    vals, vecs = np.linalg.eigh(Lq + 1e-9 * np.eye(K))
    f = vecs[:, 1]
    nz = np.flatnonzero(np.abs(f) > 1e-12)
    if len(nz) and f[nz[0]] > 0:          # sign normalisation (builder decision)
        f = -f
    order = np.argsort(f, kind="stable")
    return [groups[o] for o in order]


def _bisect_contrasts(addvec, groups):
    """Balanced binary-tree contrasts (``src/spatial.jl:204`` ``bisect_contrasts!``)."""
    if len(groups) < 2:
        return
    sz = np.cumsum([len(g) for g in groups])
    tot = sz[-1]
    h = int(np.argmin([abs(2 * sz[j] - tot) for j in range(len(groups) - 1)])) + 1
    A, B = groups[:h], groups[h:]
    addvec([i for g in A for i in g], [i for g in B for i in g])
    _bisect_contrasts(addvec, A)
    _bisect_contrasts(addvec, B)


# --------------------------------------------------------------------------------------------
# network generation
# --------------------------------------------------------------------------------------------

def _random_graph(rng, N, L):
    coords = rng.uniform(0.0, 1.0, size=(N, 2))
    d = np.sqrt(((coords[:, None, :] - coords[None, :, :]) ** 2).sum(-1))
    # Prim's minimum spanning tree
    intree = np.zeros(N, bool)
    intree[0] = True
    best = d[0].copy()
    parent = np.zeros(N, int)
    edges = set()
    for _ in range(N - 1):
        cand = np.where(intree, np.inf, best)
        j = int(np.argmin(cand))
        edges.add((min(j, parent[j]), max(j, parent[j])))
        intree[j] = True
        upd = (~intree) & (d[j] < best)
        best[upd] = d[j][upd]
        parent[upd] = j
    # shortest extra edges
    iu, ju = np.triu_indices(N, 1)
    order = np.argsort(d[iu, ju], kind="stable")
    for o in order:
        if len(edges) >= L:
            break
        e = (int(iu[o]), int(ju[o]))
        if e not in edges:
            edges.add(e)
    edges = sorted(edges)
    return coords, np.array([e[0] for e in edges], np.int32), np.array([e[1] for e in edges], np.int32)


def _countries(coords, C, iters=30):
    N = len(coords)
    centers = [0]
    dmin = np.sqrt(((coords - coords[0]) ** 2).sum(1))
    for _ in range(1, C):
        j = int(np.argmax(dmin))
        centers.append(j)
        dmin = np.minimum(dmin, np.sqrt(((coords - coords[j]) ** 2).sum(1)))
    cen = coords[centers].copy()
    lab = np.zeros(N, int)
    for _ in range(iters):
        dd = ((coords[:, None, :] - cen[None, :, :]) ** 2).sum(-1)
        lab = np.argmin(dd, 1)
        for c in range(C):
            if (lab == c).any():
                cen[c] = coords[lab == c].mean(0)
    # relabel by first appearance
    first = {}
    for l in lab:
        first.setdefault(int(l), len(first))
    return np.array([first[int(l)] for l in lab], np.int32)


def _components(N, bus0, bus1):
    parent = list(range(N))

    def find(i):
        while parent[i] != i:
            i = parent[i]
        return i
    for a, b in zip(bus0, bus1):
        ra, rb = find(int(a)), find(int(b))
        if ra != rb:
            parent[ra] = rb
    roots = list(dict.fromkeys(find(i) for i in range(N)))
    return np.array([roots.index(find(i)) for i in range(N)], np.int32)


def _logit(p):
    return math.log(p / (1.0 - p))


def make_model(N=40, L=60, T=1460, n_off=None, seed=1234, countries=None, init="uniform",
               dispatch=("OCGT",)) -> SynthModel:
    """Seeded synthetic model of the benchmark configurations (see the module docstring).
    ``dispatch`` names the dispatchable carriers, one unit of each at every node: the benchmark
    configurations have OCGT alone; a second one (e.g. ("OCGT", "CCGT")) gives nodes with several
    dispatchable units, where the pair and cell-pair selections and the Jacobian terms of the
    compensated moves come into play."""
    assert 8760 % T == 0, "T must divide 8760 (src/layout.jl:37)"
    dt = 8760.0 / T
    rng = np.random.Generator(np.random.PCG64(seed))
    n_off = (12 if N == 40 else max(1, round(0.3 * N))) if n_off is None else n_off
    C = countries if countries is not None else max(2, round(N / 4))
    coords, bus0, bus1 = _random_graph(rng, N, L)
    L = len(bus0)
    line_s = np.exp(math.log(1000.0) + 0.5 * rng.standard_normal(L))
    line_b = np.ones(L)
    country = _countries(coords, C)
    comp = _components(N, bus0, bus1)
    off_nodes = np.sort(np.argsort(coords[:, 1], kind="stable")[:n_off]).astype(np.int32)

    carriers = ["onwind", "offwind", "solar", *dispatch, "battery", "H2"]
    capex = {"onwind": 1.10e5, "offwind": 1.90e5, "solar": 0.45e5, "OCGT": 0.47e5, "CCGT": 0.90e5, "battery": 0.85e5,
             "H2": 1.20e5}
    kind, group, bus, series = [], [], [], []
    nodes_of = {"onwind": np.arange(N), "offwind": off_nodes, "solar": np.arange(N), "battery": np.arange(N),
                "H2": np.arange(N)}
    nodes_of.update({c: np.arange(N) for c in dispatch})
    # weather series: load (N), onwind (N), offwind (n_off), solar (N)  (src/energy.jl:307 wnames order)
    ser_base = {"onwind": N, "offwind": 2 * N, "solar": 2 * N + n_off}
    for gi, c in enumerate(carriers):
        for j, n in enumerate(nodes_of[c]):
            kind.append(KIND_REN if c in ser_base else (KIND_DISP if c in dispatch else KIND_STOR))
            group.append(gi)
            bus.append(int(n))
            series.append(ser_base[c] + j if c in ser_base else -1)
    kind = np.array(kind, np.int32)
    Kn = len(kind)
    mc = np.where(kind == KIND_STOR, 0.0, rng.uniform(0.0, 80.0, Kn))
    cap = np.array([capex[carriers[g]] for g in group])
    hours = np.array([6.0 if carriers[g] == "battery" else 168.0 if carriers[g] == "H2" else 0.0 for g in group])
    eta_in = np.array([0.95 if carriers[g] == "battery" else 0.70 if carriers[g] == "H2" else 0.0 for g in group])
    eta_out = np.array([0.95 if carriers[g] == "battery" else 0.55 if carriers[g] == "H2" else 0.0 for g in group])
    k0 = rng.uniform(0.0, 20000.0, Kn)

    # weather prior
    n0 = 3 * N + n_off
    sf = np.array([0] * N + [1] * N + [2] * n_off + [3] * N, np.int32)
    sn = np.concatenate([np.arange(N), np.arange(N), off_nodes, np.arange(N)]).astype(np.int32)
    load_scale = np.exp(math.log(2000.0) + 0.6 * rng.standard_normal(N))
    h = np.arange(T) * dt
    hod = np.mod(h, 24.0)
    seasonal = np.cos(2 * math.pi * h / 8760.0)
    xbar = np.zeros((n0, T))
    wscale = np.zeros(n0)
    phi, sig = 0.9, 0.3
    sig0 = sig / math.sqrt(1 - phi ** 2)
    for i in range(n0):
        n = sn[i]
        if sf[i] == 0:
            xbar[i] = load_scale[n] * (1 + 0.15 * np.sin(2 * math.pi * hod / 24.0) + 0.2 * seasonal)
            wscale[i] = 0.05 * load_scale[n] / sig0
        elif sf[i] == 1:
            xbar[i] = _logit(0.32) + 0.3 * seasonal
            wscale[i] = 1.0
        elif sf[i] == 2:
            xbar[i] = _logit(0.45) + 0.3 * seasonal
            wscale[i] = 1.0
        else:
            xbar[i] = -4.0 + 5.0 * np.maximum(0.0, np.sin(2 * math.pi * (hod - 6.0) / 24.0))
            wscale[i] = 1.0
    Kr = 2
    mu = np.zeros((Kr, n0, 3))
    shift = np.where(sf == 0, -0.005, np.where(sf == 3, -0.02, 0.06))
    mu[0, :, 0] = shift
    mu[1, :, 0] = -shift
    m = SynthModel(
        N=N, L=L, T=T, dt=dt, seed=seed, coords=coords, country=country, comp=comp,
        bus0=bus0, bus1=bus1, line_b=line_b, line_s=line_s, carriers=carriers,
        unit_kind=kind, unit_group=np.array(group, np.int32), unit_bus=np.array(bus, np.int32),
        unit_mc=mc, unit_capex=cap, unit_lo=np.zeros(Kn), unit_hi=np.full(Kn, 20000.0),
        unit_series=np.array(series, np.int32), unit_avail=np.where(kind == KIND_DISP, 1.0, 0.0),
        unit_hours=hours, unit_eta_in=eta_in, unit_eta_out=eta_out, unit_qt=np.zeros(Kn), k0=k0,
        disp=np.flatnonzero(kind == KIND_DISP).astype(np.int32), stor=np.flatnonzero(kind == KIND_STOR).astype(np.int32),
        ren=np.flatnonzero(kind == KIND_REN).astype(np.int32),
        n0=n0, series_field=sf, series_node=sn, xbar=xbar, wscale=wscale, K=Kr,
        Ptr=np.array([[0.98, 0.02], [0.02, 0.98]]), pi0=np.array([0.5, 0.5]),
        phi=np.full((Kr, n0), phi), mu=mu, sig=np.full((Kr, n0), sig), sig0=np.full(n0, sig0))
    build_tables(m)
    return m


# --------------------------------------------------------------------------------------------
# move tables (src/local.jl:44-296 GridSolver, xloc_directions, LocalModel)
# --------------------------------------------------------------------------------------------

def build_tables(m: SynthModel, cell_power: float = 1.0):
    N, L = m.N, m.L
    edges = [(int(a), int(b), float(s)) for a, b, s in zip(m.bus0, m.bus1, m.line_s)]
    parts = [np.zeros(N, np.int32), m.country, np.arange(N, dtype=np.int32)]
    # global counts (src/energy.jl:293)
    _, gcounts, _ = haar_basis(parts, np.arange(N), edges=edges)
    m.atoms = []
    # theta: partition component -> country -> node, gauge modes dropped (src/energy.jl:297)
    cols, _, _ = haar_basis([m.comp, m.country, np.arange(N)], np.arange(N), edges=edges, drop_top=True)
    m.atoms.append(_atoms(ROLE_THETA, cols, np.arange(N)))
    # one g field per dispatchable carrier, one se field per storage carrier (supports: their buses)
    for kindsel, role in ((KIND_DISP, ROLE_GEN), (KIND_STOR, ROLE_SE)):
        flat = m.disp if kindsel == KIND_DISP else m.stor
        for g in sorted(set(int(x) for x in m.unit_group[flat])):
            sel = np.array([j for j, u in enumerate(flat) if m.unit_group[u] == g], np.int32)
            sup = m.unit_bus[flat[sel]]
            cols, _, _ = haar_basis(parts, sup, edges=edges)
            m.atoms.append(_atoms(role, cols, sel))
    # node incidence
    nl = [[] for _ in range(N)]
    for e in range(L):
        nl[m.bus0[e]].append(e)
        nl[m.bus1[e]].append(e)
    m.nodelines_ptr, m.nodelines = _csr(nl)
    # dispatchable and storage units per node (src/local.jl:257,285)
    m.units_ptr, m.units_at = _csr([[j for j, u in enumerate(m.disp) if m.unit_bus[u] == n] for n in range(N)])
    m.stor_ptr, m.stor_at = _csr([[j for j, u in enumerate(m.stor) if m.unit_bus[u] == n] for n in range(N)])
    # cell moves: partition levels resolved at the complete level (src/local.jl:265-283)
    qlev = len(gcounts)
    cells_per_level = []
    for q in range(qlev):
        lab = [tuple(int(parts[p][n]) for p in range(q + 1)) for n in range(N)]
        keys = list(dict.fromkeys(lab))
        cu = [[] for _ in keys]
        for j, u in enumerate(m.disp):               # injecting fields: the dispatchable generators
            cu[keys.index(lab[m.unit_bus[u]])].append(j)
        cells_per_level.append(cu)
    qw = np.array([float(len(cu)) ** cell_power for cu in cells_per_level])
    m.qcum = np.cumsum(qw) / qw.sum()
    flat_cells = [c for cu in cells_per_level for c in cu]
    m.cell_ptr, m.cell_units = _csr(flat_cells)
    m.cell_level_ptr = np.cumsum([0] + [len(cu) for cu in cells_per_level]).astype(np.int32)
    # grid solver and xloc templates
    _grid_tables(m, nl)


def _atoms(role, cols, idxmap):
    ptr = [0]
    idx, val = [], []
    for rows, vals in cols:
        idx.extend(int(idxmap[r]) for r in rows)
        val.extend(vals)
        ptr.append(len(idx))
    return Atoms(role, np.array(ptr, np.int32), np.array(idx, np.int32), np.array(val, float))


def _csr(lists):
    ptr = np.cumsum([0] + [len(x) for x in lists]).astype(np.int32)
    dat = np.array([v for x in lists for v in x], np.int32)
    return ptr, dat


def _grid_tables(m: SynthModel, nl):
    N = m.N
    # GridSolver (src/local.jl:52): per component, the Laplacian grounded at its first node
    Z = np.zeros((N, N))
    for c in range(int(m.comp.max()) + 1):
        nd = np.flatnonzero(m.comp == c)
        if len(nd) < 2:
            continue
        loc = {int(n): j for j, n in enumerate(nd[1:])}
        k = len(nd) - 1
        A = np.zeros((k, k))
        for a, b, w in zip(m.bus0, m.bus1, m.line_b):
            if m.comp[a] != c:
                continue
            ia, ib = loc.get(int(a), -1), loc.get(int(b), -1)
            if ia >= 0:
                A[ia, ia] += w
            if ib >= 0:
                A[ib, ib] += w
            if ia >= 0 and ib >= 0:
                A[ia, ib] -= w
                A[ib, ia] -= w
        Ainv = np.linalg.inv(A)
        for n in nd[1:]:
            for i in nd[1:]:
                Z[i, n] = Ainv[loc[int(i)], loc[int(n)]]
    m.reroute = Z
    # xloc_directions with rp = 1, rb = 0 (src/local.jl:122): partners are the neighbours
    nbr = [sorted({int(m.bus1[e]) if m.bus0[e] == n else int(m.bus0[e]) for e in nl[n]} - {n}) for n in range(N)]
    part, xn, xv, lkn, lkg = [], [], [], [], []
    for n in range(N):
        part.append(nbr[n])
        for mm in nbr[n]:
            B = sorted({n, mm})
            compsize = int((m.comp == m.comp[n]).sum())
            if len(B) >= compsize:               # whole component: exact re-routing
                x = Z[:, n] - Z[:, mm]
                nd = np.flatnonzero(m.comp == m.comp[n])
                keep = [int(i) for i in nd if abs(x[i]) >= 1e-15]
                xn.append(keep)
                xv.append([float(x[i]) for i in keep])
                lkn.append([])
                lkg.append([])
                continue
            loc = {i: j for j, i in enumerate(B)}
            Lb = np.zeros((len(B), len(B)))
            for i in B:
                for e in nl[i]:
                    a, b = int(m.bus0[e]), int(m.bus1[e])
                    o = b if a == i else a
                    w = m.line_b[e]
                    Lb[loc[i], loc[i]] += w
                    if o in loc:
                        Lb[loc[i], loc[o]] -= w
            rhs = np.zeros(len(B))
            rhs[loc[n]] += 1.0
            rhs[loc[mm]] -= 1.0
            th = np.linalg.solve(Lb, rhs)
            keep = [j for j in range(len(B)) if abs(th[j]) >= 1e-15]
            xn.append([B[j] for j in keep])
            xv.append([float(th[j]) for j in keep])
            ln, lg = [], []
            for q, i in enumerate(B):
                for e in nl[i]:
                    a, b = int(m.bus0[e]), int(m.bus1[e])
                    o = b if a == i else a
                    if o in loc:
                        continue
                    if o not in ln:
                        ln.append(o)
                        lg.append(0.0)
                    lg[ln.index(o)] -= m.line_b[e] * th[q]
            p = np.argsort(ln, kind="stable")
            lkn.append([ln[j] for j in p])
            lkg.append([lg[j] for j in p])
    m.xpart_ptr, m.xpart = _csr(part)
    m.xnod_ptr, m.xnod = _csr(xn)
    m.xval = np.array([v for x in xv for v in x], float)
    m.xlk_ptr, m.xlkn = _csr(lkn)
    m.xlkg = np.array([v for x in lkg for v in x], float)


# --------------------------------------------------------------------------------------------
# weather draws and the start state
# --------------------------------------------------------------------------------------------

def datamap(m: SynthModel, X):
    """Weather data map per series: load (x)+, availability logistic(x) (builder decision)."""
    out = np.empty_like(X)
    ld = m.series_field == 0
    out[ld] = np.maximum(X[ld], 0.0)
    out[~ld] = 1.0 / (1.0 + np.exp(-X[~ld]))
    return out


def sample_weather(m: SynthModel, rng):
    """Exact draw (regimes, anomaly z) from the prior (``src/weather.jl:461`` ``sample_weather``)."""
    T, n0 = m.T, m.n0
    reg = np.zeros(T, np.int32)
    reg[0] = rng.choice(m.K, p=m.pi0)
    for t in range(1, T):
        reg[t] = rng.choice(m.K, p=m.Ptr[reg[t - 1]])
    e = rng.standard_normal((n0, T))
    z = np.zeros((n0, T))
    z[:, 0] = m.sig0 * e[:, 0]
    for t in range(1, T):
        c, cs, sn = 1.0, math.cos(2 * math.pi * (t + 1) / T), math.sin(2 * math.pi * (t + 1) / T)
        k = reg[t]
        mean = m.phi[k] * z[:, t - 1] + c * m.mu[k, :, 0] + cs * m.mu[k, :, 1] + sn * m.mu[k, :, 2]
        z[:, t] = mean + m.sig[k] * e[:, t]
    return reg, z


def weather_nodes(m: SynthModel, z):
    """Raw node weather X = xbar + scale z (``src/weather.jl:410``), per series."""
    return m.xbar + m.wscale[:, None] * z


@dataclass
class ReplicaState:
    """Node-valued state of R replicas, (series/unit, T, R) arrays with the replica index fastest."""
    theta: np.ndarray   # [N, T, R]
    g: np.ndarray       # [D, T, R]
    e: np.ndarray       # [S, T, R]
    z: np.ndarray       # [n0, T, R] weather anomaly
    reg: np.ndarray     # [T, R] regimes
    k: np.ndarray       # [Kunits]


def sample_weather_batch(m: SynthModel, R: int, rng):
    """Exact prior draws of R replicas at once (the recursion of ``src/weather.jl:461``
    ``sample_weather``, vectorised over replicas): regimes [T, R] and anomalies [n0, T, R]."""
    T, n0 = m.T, m.n0
    reg = np.zeros((T, R), np.int32)
    cum0 = np.cumsum(m.pi0)
    cumP = np.cumsum(m.Ptr, axis=1)
    reg[0] = np.minimum(np.searchsorted(cum0, rng.random(R), side="left"), m.K - 1)
    u = rng.random((T, R))
    for t in range(1, T):
        reg[t] = np.minimum((u[t][:, None] > cumP[reg[t - 1]]).sum(1), m.K - 1)
    z = np.zeros((n0, T, R))
    z[:, 0, :] = m.sig0[:, None] * rng.standard_normal((n0, R))
    cols = np.arange(n0)
    for t in range(1, T):
        e = rng.standard_normal((n0, R))
        cs, sn = math.cos(2 * math.pi * (t + 1) / T), math.sin(2 * math.pi * (t + 1) / T)
        k = reg[t]
        mean = (m.phi[k].T * z[:, t - 1, :] + m.mu[k, :, 0].T + cs * m.mu[k, :, 1].T + sn * m.mu[k, :, 2].T)
        z[:, t, :] = mean + m.sig[k].T * e
    del cols
    return reg, z


def initial_state(m: SynthModel, R: int, seed: int = 7) -> ReplicaState:
    """Start state: independent prior weather draws per replica, zero angles, OCGT covering the
    residual load after renewables, storage half full (a heuristic interior start in the spirit of
    ``src/run.jl:470`` ``heuristic_start``)."""
    T = m.T
    rng = np.random.Generator(np.random.PCG64([seed, R]))
    reg, z = sample_weather_batch(m, R, rng)
    X = m.xbar[:, :, None] + m.wscale[:, None, None] * z
    W = np.empty_like(X)
    ld = m.series_field == 0
    W[ld] = np.maximum(X[ld], 0.0)
    W[~ld] = 1.0 / (1.0 + np.exp(-X[~ld]))
    res = W[:m.N].copy()
    for u in m.ren:
        res[m.unit_bus[u]] -= W[m.unit_series[u]] * m.k0[u]
    g = np.zeros((m.D, T, R))
    for j, u in enumerate(m.disp):
        kap = m.unit_avail[u] * m.k0[u]
        g[j] = np.clip(res[m.unit_bus[u]] / max(kap, 1e-9), 0.0, 1.0) if kap > 0 else 0.0
    return ReplicaState(theta=np.zeros((m.N, T, R)), g=g, e=np.full((m.S, T, R), 0.5), z=z, reg=reg,
                        k=m.k0.copy())
