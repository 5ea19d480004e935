"""Process definitions: channel trees and mapping tables in Whizard's layout.

A process holds, per channel, the tables the reference's C-ABI takes
(whizard_gpu_phs.cpp:57-87) and its .ref files store (file_input.cpp:183-250):

* ``d1``, ``d2``, ``has_children``: int32 ``[n_channels, N_PRT]`` indexed by
  Whizard code - 1, holding daughter codes (0 = none).  Outgoing particle j has
  code 2**j, a branch's code is the OR of its leaves, the root is 2**n_out - 1,
  N_PRT = 2**(n_in+n_out) - 1.
* ``friends``: int32 ``[n_channels, N_PRT]``.
* ``map_ids``, ``map_masses``, ``map_widths``: ``[n_channels, N_PRT_OUT]``
  indexed by code - 1, N_PRT_OUT = 2**n_out - 1.
* ``flv_masses``, ``flv_widths``: ``[n_in + n_out]`` (incoming first).

The builders below give the benchmark workloads: e+e- -> W+W- -> 4f at 500 GeV,
e+e- -> t tbar -> 6f at 1 TeV, the 2 -> 6 massless caterpillar at 13 TeV, and
seeded random multi-channel sets for batching.
"""
from __future__ import annotations

from dataclasses import dataclass, field
from typing import Dict, List, Sequence, Tuple, Union

import numpy as np

MAP_NO = 0
MAP_SCHANNEL = 1
MAP_TCHANNEL = 2
MAP_UCHANNEL = 3
MAP_RADIATION = 4
MAP_COLLINEAR = 5
MAP_INFRARED = 6
MAP_STEP_E = 11
MAP_STEP_H = 12
MAP_ONSHELL = 99
MAP_IDS = (MAP_NO, MAP_SCHANNEL, MAP_TCHANNEL, MAP_UCHANNEL, MAP_RADIATION, MAP_COLLINEAR,
           MAP_INFRARED, MAP_STEP_E, MAP_STEP_H)

M_ELECTRON = 0.000510997

Tree = Union[int, Tuple["Tree", "Tree"]]


@dataclass
class Process:
    """One Whizard process: n_channels trees over the same external particles."""

    n_in: int
    n_out: int
    d1: np.ndarray
    d2: np.ndarray
    has_children: np.ndarray
    friends: np.ndarray
    map_ids: np.ndarray
    map_masses: np.ndarray
    map_widths: np.ndarray
    flv_masses: np.ndarray
    flv_widths: np.ndarray
    n_x: int = 0            # x stride per event (>= 3*n_out - 4)
    name: str = ""
    sqrts: float = 0.0      # nominal collision energy of the workload

    @property
    def n_channels(self) -> int:
        return int(self.d1.shape[0])

    @property
    def n_prt(self) -> int:
        return (1 << (self.n_in + self.n_out)) - 1

    @property
    def n_prt_out(self) -> int:
        return (1 << self.n_out) - 1

    @property
    def n_x_used(self) -> int:
        return 3 * self.n_out - 4

    def subset(self, channels: Sequence[int]) -> "Process":
        ch = np.asarray(channels, dtype=np.int64)
        return Process(self.n_in, self.n_out, self.d1[ch].copy(), self.d2[ch].copy(),
                       self.has_children[ch].copy(), self.friends[ch].copy(),
                       self.map_ids[ch].copy(), self.map_masses[ch].copy(),
                       self.map_widths[ch].copy(), self.flv_masses.copy(),
                       self.flv_widths.copy(), self.n_x, self.name, self.sqrts)


def _tree_code(t: Tree) -> int:
    if isinstance(t, int):
        return 1 << t
    return _tree_code(t[0]) | _tree_code(t[1])


def process_from_trees(trees: Sequence[Tree], maps: Sequence[Dict[int, Tuple[int, float, float]]],
                       flv_masses: Sequence[float], flv_widths: Sequence[float] | None = None,
                       n_in: int = 2, n_x: int = 0, name: str = "", sqrts: float = 0.0) -> Process:
    """Build a process from nested-tuple trees over leaf indices 0..n_out-1.

    ``maps[c]`` maps a branch code to (map_id, mass, width); codes not listed get
    MAP_NO with zero mass and width.
    """
    n_out = len(flv_masses) - n_in
    n_prt = (1 << (n_in + n_out)) - 1
    n_prt_out = (1 << n_out) - 1
    nc = len(trees)
    d1 = np.zeros((nc, n_prt), np.int32)
    d2 = np.zeros((nc, n_prt), np.int32)
    hc = np.zeros((nc, n_prt), np.int32)
    mid = np.zeros((nc, n_prt_out), np.int32)
    mm = np.zeros((nc, n_prt_out), np.float64)
    mw = np.zeros((nc, n_prt_out), np.float64)
    for c, t in enumerate(trees):
        if _tree_code(t) != n_prt_out:
            raise ValueError(f"channel {c}: tree does not cover all {n_out} outgoing particles")

        def walk(node: Tree) -> int:
            if isinstance(node, int):
                return 1 << node
            a, b = walk(node[0]), walk(node[1])
            code = a | b
            lo, hi = (a, b) if a < b else (b, a)
            d1[c, code - 1], d2[c, code - 1], hc[c, code - 1] = lo, hi, 1
            return code

        walk(t)
        for code, (typ, m, w) in maps[c].items():
            mid[c, code - 1], mm[c, code - 1], mw[c, code - 1] = typ, m, w
    fw = np.zeros(n_in + n_out) if flv_widths is None else np.asarray(flv_widths, np.float64)
    nx = n_x if n_x else 3 * n_out - 4
    return Process(n_in, n_out, d1, d2, hc, np.zeros_like(d1), mid, mm, mw,
                   np.asarray(flv_masses, np.float64), fw, nx, name, sqrts)


def ww() -> Process:
    """e+e- -> W+W- -> 4 massless fermions at sqrt(s) = 500 GeV; both W Breit-Wigner."""
    mw_, gw = 80.419, 2.048
    tree = ((0, 1), (2, 3))
    maps = {0b0011: (MAP_SCHANNEL, mw_, gw), 0b1100: (MAP_SCHANNEL, mw_, gw)}
    return process_from_trees([tree], [maps], [M_ELECTRON, M_ELECTRON, 0, 0, 0, 0],
                              n_x=8, name="ee_WW_4f_500GeV", sqrts=500.0)


def tt() -> Process:
    """e+e- -> t tbar -> b (l+ nu) bbar (q q') at sqrt(s) = 1 TeV, massive b quarks.

    Outgoing order: b, l+, nu, bbar, q, q'.  t/tbar Breit-Wigner m=173.0 G=1.5,
    W+/W- Breit-Wigner m=80.419 G=2.048.
    """
    mt, gt, mw_, gw, mb = 173.0, 1.5, 80.419, 2.048, 4.7
    tree = ((0, (1, 2)), (3, (4, 5)))
    maps = {0b000111: (MAP_SCHANNEL, mt, gt), 0b111000: (MAP_SCHANNEL, mt, gt),
            0b000110: (MAP_SCHANNEL, mw_, gw), 0b110000: (MAP_SCHANNEL, mw_, gw)}
    return process_from_trees([tree], [maps], [M_ELECTRON, M_ELECTRON, mb, 0, 0, mb, 0, 0],
                              n_x=14, name="ee_tt_6f_1TeV", sqrts=1000.0)


def precision() -> Process:
    """2 -> 6 massless partons at 13 TeV: a 5-level caterpillar tree with the log
    (infrared) msq mapping, m = 10 GeV, and uniform cos(theta) on every internal
    branch; x stride 16 (14 used)."""
    tree: Tree = 4
    tree = (tree, 5)
    for leaf in (3, 2, 1, 0):
        tree = (leaf, tree)
    maps = {}

    def collect(node: Tree) -> int:
        if isinstance(node, int):
            return 1 << node
        code = collect(node[0]) | collect(node[1])
        maps[code] = (MAP_INFRARED, 10.0, 0.0)
        return code

    collect(tree)
    return process_from_trees([tree], [maps], [0.0] * 8, n_x=16, name="pp_6j_13TeV_infrared",
                              sqrts=13000.0)


def random_tree(rng: np.random.Generator, leaves: List[int]) -> Tree:
    if len(leaves) == 1:
        return int(leaves[0])
    k = int(rng.integers(1, len(leaves)))
    perm = [int(v) for v in rng.permutation(leaves)]
    return (random_tree(rng, sorted(perm[:k])), random_tree(rng, sorted(perm[k:])))


def random_process(rng: np.random.Generator, n_out: int, n_channels: int, sqrts: float = 1000.0,
                   name: str = "") -> Process:
    """n_channels random trees over n_out outgoing particles of random masses, with
    per-branch mappings drawn from Breit-Wigner (m in 10-500 GeV, scaled with the
    branch's number of leaves; G/m in 0.005-0.05),
    massless log/collinear (mapping mass 1-20 GeV), t-channel exponential (mapping mass
    1-20 GeV) and uniform."""
    leaf_masses = rng.choice([0.0, 0.0, 0.0, 0.105658, 1.5, 4.7], size=n_out)
    trees, maps = [], []
    for _ in range(n_channels):
        t = random_tree(rng, list(range(n_out)))
        mp: Dict[int, Tuple[int, float, float]] = {}

        def assign(node: Tree, depth: int) -> int:
            if isinstance(node, int):
                return 1 << node
            code = assign(node[0], depth + 1) | assign(node[1], depth + 1)
            if depth == 0:
                mp[code] = (MAP_NO, 0.0, 0.0)
                return code
            # t-channel and unmapped branches hang off the root (they sample msq up to
            # the kinematic limit); deeper branches are resonances or collinear splittings
            if depth == 1:
                kind = rng.choice(4, p=[0.5, 0.2, 0.15, 0.15])
            else:
                kind = rng.choice(2, p=[0.7, 0.3])
            if kind == 0:
                # resonance masses shrink with the branch's share of the final state, so
                # that nested Breit-Wigners are kinematically compatible
                share = bin(code).count("1") / n_out
                m = float(np.clip(rng.uniform(0.2, 0.6) * share * sqrts, 10.0, 500.0))
                mp[code] = (MAP_SCHANNEL, m, m * float(rng.uniform(0.005, 0.05)))
            elif kind == 1:
                mp[code] = (int(rng.choice([MAP_COLLINEAR, MAP_INFRARED])),
                            float(rng.uniform(1.0, 20.0)), 0.0)
            elif kind == 2:
                mp[code] = (MAP_TCHANNEL, float(rng.uniform(1.0, 20.0)), 0.0)
            else:
                mp[code] = (MAP_NO, 0.0, 0.0)
            return code

        assign(t, 0)
        trees.append(t)
        maps.append(mp)
    flv = [M_ELECTRON, M_ELECTRON] + [float(m) for m in leaf_masses]
    return process_from_trees(trees, maps, flv, name=name, sqrts=sqrts)


def nested_resonances(n_out: int, sqrts: float = 1000.0, per_particle: float = 25.0) -> Process:
    """Three channels over n_out massless particles -- a balanced tree, a caterpillar and
    the balanced tree over the reversed particles -- whose internal branches below the root
    are Breit-Wigner resonances of per_particle GeV per particle below them (width 2 %),
    so that nested resonances are kinematically compatible: the largest trees the API
    takes with a sizeable ok fraction."""
    def balanced(leaves):
        if len(leaves) == 1:
            return leaves[0]
        h = len(leaves) // 2
        return (balanced(leaves[:h]), balanced(leaves[h:]))

    def caterpillar(leaves):
        t = leaves[0]
        for k in leaves[1:]:
            t = (t, k)
        return t

    def resonances(t, mp, depth=0):
        if isinstance(t, int):
            return 1 << t
        code = resonances(t[0], mp, depth + 1) | resonances(t[1], mp, depth + 1)
        if depth:
            m = per_particle * bin(code).count("1")
            mp[code] = (MAP_SCHANNEL, m, 0.02 * m)
        return code

    leaves = list(range(n_out))
    trees = [balanced(leaves), caterpillar(leaves), balanced(leaves[::-1])]
    maps = []
    for t in trees:
        mp: Dict[int, Tuple[int, float, float]] = {}
        resonances(t, mp)
        maps.append(mp)
    return process_from_trees(trees, maps, [M_ELECTRON, M_ELECTRON] + [0.0] * n_out,
                              name=f"nested_resonances_{n_out}", sqrts=sqrts)


def batched(seed: int = 2024, n_channels: int = 64, total_events: int = 1 << 24,
            sqrts: float = 1000.0) -> Tuple[List[Process], np.ndarray]:
    """The batched workload: n_channels single-channel processes with 3-8 outgoing
    particles, and power-law (exponent 1.5) event counts summing to total_events.

    Returns (processes, counts); channel i is process i."""
    rng = np.random.default_rng(seed)
    procs = []
    for i in range(n_channels):
        n_out = int(rng.integers(3, 9))
        procs.append(random_process(rng, n_out, 1, sqrts, name=f"batch{i}_n{n_out}"))
    w = np.arange(1, n_channels + 1, dtype=np.float64) ** -1.5
    w = w[rng.permutation(n_channels)]
    counts = np.floor(w / w.sum() * total_events).astype(np.int64)
    counts = np.maximum(counts, 1)
    counts[int(np.argmax(counts))] += total_events - int(counts.sum())
    return procs, counts
