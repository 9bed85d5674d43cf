"""n2p2 potential files: reading, and writing seeded synthetic potentials.

The reference's ForceNNP::init_coeff loads an n2p2 potential directory
(src/force_types/force_nnp_cabana_neigh_impl.h:41-66): ``input.nn``
(settings and symmetry functions), ``scaling.data`` (per-function min, max,
mean, sigma) and ``weights.%03d.data`` (one file per element, named by
atomic number).  The formats are n2p2 v2.0.1's, as used by the reference's
fixture ``input/nnp``.

Symmetry functions are kept in n2p2's canonical order, which is also the
row order of ``scaling.data``: radial (type 2) before angular (type 3), then
by cutoff, the neighbour element(s), eta, zeta, lambda and rs.  The
reference fixture's ``scaling.data`` follows exactly this order (its rows
alternate the two lambdas within each zeta and climb zeta within each eta,
while its ``input.nn`` lists zeta as 1, 16, 2, 4).

Several elements follow n2p2's element map: elements are indexed in order
of atomic number (the index of ``scaling.data``'s first column, and the atom
type CabanaMD passes, src/force_types/force_nnp_cabana_neigh_impl.h:93-98),
neighbour elements order by atomic number too, and an angular function's
two neighbour elements are stored lighter first.  No reference test or
fixture exercises more than one element, so this ordering is restated from
n2p2's documented conventions and is unpinned.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field
from pathlib import Path

import numpy as np

ELEMENTS = ("H He Li Be B C N O F Ne Na Mg Al Si P S Cl Ar K Ca Sc Ti V Cr Mn Fe Co Ni Cu Zn "
            "Ga Ge As Se Br Kr Rb Sr Y Zr Nb Mo Tc Ru Rh Pd Ag Cd In Sn Sb Te I Xe Cs Ba La "
            "Ce Pr Nd Pm Sm Eu Gd Tb Dy Ho Er Tm Yb Lu Hf Ta W Re Os Ir Pt Au Hg Tl Pb Bi").split()


def atomic_number(symbol: str) -> int:
    return ELEMENTS.index(symbol) + 1


@dataclass
class SymFn:
    type: int
    elem: str
    neighbors: tuple
    eta: float
    rs: float = 0.0
    lam: float = 0.0
    zeta: float = 0.0
    rc: float = 0.0

    def key(self):
        z = sorted(atomic_number(e) for e in self.neighbors)
        z += [0] * (2 - len(z))
        return (self.type, self.rc, z[0], z[1], self.eta, self.zeta, self.lam, self.rs)


@dataclass
class Potential:
    elements: list
    atom_energy: dict
    cutoff_type: int
    smin: float
    smax: float
    nodes: list           # hidden + output node counts, e.g. [25, 25, 1]
    activations: str      # one code per layer after the input, e.g. "ppl"
    symfns: dict          # element -> list[SymFn] in canonical order
    gmin: dict            # element -> np.ndarray
    gmax: dict
    W: dict = field(default_factory=dict)  # element -> list of (nodes[l] x nodes[l-1])
    b: dict = field(default_factory=dict)
    settings: dict = field(default_factory=dict)

    def nsf(self, elem):
        return len(self.symfns[elem])


def _parse_input(path: Path) -> dict:
    kw = {}
    sfs = []
    for line in path.read_text().splitlines():
        t = line.split("#")[0].split()
        if not t:
            continue
        if t[0] == "symfunction_short":
            elem, typ = t[1], int(t[2])
            if typ == 2:
                sfs.append(SymFn(2, elem, (t[3],), float(t[4]), rs=float(t[5]), rc=float(t[6])))
            elif typ == 3:
                rs = float(t[9]) if len(t) > 9 else 0.0
                pair = tuple(sorted((t[3], t[4]), key=atomic_number))
                sfs.append(SymFn(3, elem, pair, float(t[5]), lam=float(t[6]),
                                 zeta=float(t[7]), rc=float(t[8]), rs=rs))
            else:
                raise ValueError(f"symmetry function type {typ} not supported")
        elif t[0] == "atom_energy":
            kw.setdefault("atom_energy", {})[t[1]] = float(t[2])
        else:
            kw[t[0]] = t[1:]
    kw["symfns"] = sfs
    return kw


def read_potential(directory) -> Potential:
    d = Path(directory)
    kw = _parse_input(d / "input.nn")
    elements = sorted(kw["elements"], key=atomic_number)
    if int(kw["number_of_elements"][0]) != len(elements):
        raise ValueError("number_of_elements does not match elements")
    nodes = [int(v) for v in kw["global_nodes_short"]] + [1]
    acts = "".join(kw["global_activation_short"])
    if len(acts) != len(nodes):
        raise ValueError("global_activation_short needs one code per layer")
    symfns = {e: sorted([s for s in kw["symfns"] if s.elem == e], key=SymFn.key)
              for e in elements}
    # scaling.data: element index, function index, min, max, mean, sigma
    gmin = {e: np.zeros(len(symfns[e])) for e in elements}
    gmax = {e: np.zeros(len(symfns[e])) for e in elements}
    for line in (d / "scaling.data").read_text().splitlines():
        t = line.split()
        if not t or t[0].startswith("#") or len(t) < 4:
            continue
        ei, si = int(t[0]) - 1, int(t[1]) - 1
        e = elements[ei]
        gmin[e][si] = float(t[2])
        gmax[e][si] = float(t[3])
    pot = Potential(elements, kw.get("atom_energy", {}), int(kw["cutoff_type"][0]),
                    float(kw.get("scale_min_short", ["0"])[0]),
                    float(kw.get("scale_max_short", ["1"])[0]), nodes, acts, symfns, gmin, gmax,
                    settings=kw)
    for e in elements:
        layers = [len(symfns[e])] + nodes
        W = [np.zeros((layers[l], layers[l - 1])) for l in range(1, len(layers))]
        b = [np.zeros(layers[l]) for l in range(1, len(layers))]
        for line in (d / f"weights.{atomic_number(e):03d}.data").read_text().splitlines():
            t = line.split()
            if not t or t[0].startswith("#"):
                continue
            val = float(t[0])
            if t[1] == "a":  # value a index l_from n_from l_to n_to (1-based nodes)
                lf, nf, lt, nt = int(t[3]), int(t[4]), int(t[5]), int(t[6])
                if lt != lf + 1:
                    raise ValueError("weight does not connect adjacent layers")
                W[lf][nt - 1, nf - 1] = val
            elif t[1] == "b":  # value b index layer node
                l, nd = int(t[3]), int(t[4])
                b[l - 1][nd - 1] = val
        pot.W[e] = W
        pot.b[e] = b
    return pot


def write_potential(directory, pot: Potential) -> None:
    """Write input.nn, scaling.data and weights.%03d.data for pot."""
    d = Path(directory)
    d.mkdir(parents=True, exist_ok=True)
    if list(pot.elements) != sorted(pot.elements, key=atomic_number):
        raise ValueError("elements must be in order of atomic number")
    lines = [f"number_of_elements {len(pot.elements)}",
             "elements " + " ".join(pot.elements)]
    for e in pot.elements:
        lines.append(f"atom_energy {e} {pot.atom_energy.get(e, 0.0)!r}")
    lines += [f"cutoff_type {pot.cutoff_type}", "scale_symmetry_functions",
              f"scale_min_short {pot.smin!r}", f"scale_max_short {pot.smax!r}",
              f"global_hidden_layers_short {len(pot.nodes) - 1}",
              "global_nodes_short " + " ".join(str(v) for v in pot.nodes[:-1]),
              "global_activation_short " + " ".join(pot.activations)]
    for e in pot.elements:
        for s in pot.symfns[e]:
            if s.type == 2:
                lines.append(f"symfunction_short {e} 2 {s.neighbors[0]} {s.eta!r} {s.rs!r} "
                             f"{s.rc!r}")
            else:
                lines.append(f"symfunction_short {e} 3 {s.neighbors[0]} {s.neighbors[1]} "
                             f"{s.eta!r} {int(s.lam)} {s.zeta!r} {s.rc!r}")
    (d / "input.nn").write_text("\n".join(lines) + "\n")
    sl = []
    for ei, e in enumerate(pot.elements):
        for si in range(pot.nsf(e)):
            lo, hi = pot.gmin[e][si], pot.gmax[e][si]
            sl.append(f"{ei + 1:4d} {si + 1:4d} {lo:.17e} {hi:.17e} {0.5 * (lo + hi):.17e} "
                      f"{0.0:.17e}")
    (d / "scaling.data").write_text("\n".join(sl) + "\n")
    for e in pot.elements:
        out = []
        k = 1
        W, b = pot.W[e], pot.b[e]
        for l in range(len(W)):
            for nf in range(W[l].shape[1]):
                for nt in range(W[l].shape[0]):
                    out.append(f"{W[l][nt, nf]:.17e} a {k:9d} {l:5d} {nf + 1:5d} {l + 1:5d} "
                               f"{nt + 1:5d}")
                    k += 1
            for nt in range(b[l].shape[0]):
                out.append(f"{b[l][nt]:.17e} b {k:9d} {l + 1:5d} {nt + 1:5d}")
                k += 1
        (d / f"weights.{atomic_number(e):03d}.data").write_text("\n".join(out) + "\n")


def synthetic_cu_potential(seed: int = 2024, rc: float = 6.0) -> Potential:
    """The Cu-like potential of the NNP workloads: 8 radial G2 (rs 0) + 24
    angular G3 (eta x zeta x lambda), cosine cutoff rc, 32-25-25-1 softplus
    hidden layers and a linear output, weights N(0, 1/fan_in) from seed, zero
    biases.  Scaling bounds are left at [0, 1] until fitted to a state
    (fit_scaling)."""
    e = "Cu"
    sfs = [SymFn(2, e, (e,), eta, rs=0.0, rc=rc)
           for eta in (0.001, 0.01, 0.03, 0.06, 0.15, 0.3, 0.6, 1.5)]
    sfs += [SymFn(3, e, (e, e), eta, lam=lam, zeta=zeta, rc=rc)
            for eta in (0.001, 0.01, 0.05) for zeta in (1.0, 2.0, 4.0, 16.0)
            for lam in (-1.0, 1.0)]
    sfs = sorted(sfs, key=SymFn.key)
    nodes = [25, 25, 1]
    rng = np.random.default_rng(seed)
    layers = [len(sfs)] + nodes
    W = [rng.normal(0.0, 1.0 / math.sqrt(layers[l - 1]), size=(layers[l], layers[l - 1]))
         for l in range(1, len(layers))]
    b = [np.zeros(layers[l]) for l in range(1, len(layers))]
    n = len(sfs)
    return Potential([e], {e: 0.0}, 1, -1.0, 1.0, nodes, "ppl", {e: sfs},
                     {e: np.zeros(n)}, {e: np.ones(n)}, {e: W}, {e: b})


def fit_scaling(pot: Potential, elem: str, G: np.ndarray) -> None:
    """Set Gmin/Gmax from raw symmetry functions of a reference state (the
    workloads' "min/max over step 0").  Constant functions get a unit
    range so the scaling stays finite."""
    lo = G.min(axis=0)
    hi = G.max(axis=0)
    same = hi - lo <= 1e-12 * np.maximum(1.0, np.abs(hi))
    hi = np.where(same, lo + 1.0, hi)
    pot.gmin[elem] = lo
    pot.gmax[elem] = hi


def synthetic_binary_potential(seed: int = 7, elements=("Ni", "Cu"), rc: float = 6.0) -> Potential:
    """A two-element potential for the multi-element paths: per centre
    element, G2 for each neighbour element (4 etas) and G3 for each
    unordered neighbour pair (2 etas x zeta 1, 4 x lambda +-1), cosine cutoff
    rc, 16-16-1 tanh/tanh/linear layers, weights N(0, 1/fan_in) from seed,
    small random biases.  Scaling bounds are left at [0, 1] until fitted."""
    elems = sorted(elements, key=atomic_number)
    rng = np.random.default_rng(seed)
    symfns, gmin, gmax, W, b = {}, {}, {}, {}, {}
    nodes = [16, 16, 1]
    pairs = [(a, c) for k, a in enumerate(elems) for c in elems[k:]]
    for e in elems:
        sfs = [SymFn(2, e, (n,), eta, rs=0.0, rc=rc)
               for n in elems for eta in (0.004, 0.04, 0.2, 0.8)]
        sfs += [SymFn(3, e, pr, eta, lam=lam, zeta=zeta, rc=rc)
                for pr in pairs for eta in (0.005, 0.05) for zeta in (1.0, 4.0)
                for lam in (-1.0, 1.0)]
        sfs = sorted(sfs, key=SymFn.key)
        symfns[e] = sfs
        layers = [len(sfs)] + nodes
        W[e] = [rng.normal(0.0, 1.0 / math.sqrt(layers[l - 1]), size=(layers[l], layers[l - 1]))
                for l in range(1, len(layers))]
        b[e] = [rng.normal(0.0, 0.1, size=layers[l]) for l in range(1, len(layers))]
        gmin[e] = np.zeros(len(sfs))
        gmax[e] = np.ones(len(sfs))
    energies = {e: -0.5 * (k + 1) for k, e in enumerate(elems)}
    return Potential(elems, energies, 1, -1.0, 1.0, nodes, "ttl", symfns, gmin, gmax, W, b)

