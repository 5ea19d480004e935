"""Reader for Whizard's phase-space reference files (.ref).

Format, as the reference's reader takes it (file_input.cpp:163-324,
file_input.h:29-30):

* 6 header lines ``key value``: n_channels, n_in, n_out, n_trees, n_groves, n_x.
* per tree, 7 lines: ``daughters1``/``daughters2``/``haschildren`` with N_PRT
  Whizard codes (daughter codes, 0 = none), ``hasfriends`` with ONE flag, and
  ``mappings``/``map_masses``/``map_widths`` with N_PRT_OUT entries.
* ``flv_masses`` and ``flv_widths`` with n_in + n_out entries.
* per event: ``channel c`` (1-based), ``x: ...`` (n_x values), n_in + n_out
  momentum lines (incoming first), ``Volume: v``, ``ok: k``, and
  ``all_factors: ...`` (one per channel).
"""
from __future__ import annotations

from dataclasses import dataclass
from typing import List

import numpy as np

from .processes import Process


@dataclass
class RefEvents:
    channel: np.ndarray      # int32 [n], 0-based
    x: np.ndarray            # float64 [n, n_x]
    p_in: np.ndarray         # float64 [n, n_in, 4]
    p_out: np.ndarray        # float64 [n, n_out, 4]
    volume: np.ndarray       # float64 [n]
    ok: np.ndarray           # int8 [n]
    all_factors: np.ndarray  # float64 [n, n_channels]


def friends_from_trees(n_out: int, d1, d2, has_children, flags) -> np.ndarray:
    """Friend table [n_trees, N_PRT] (Whizard code of the paired incoming particle, 0 =
    none) from the trees of a .ref file, which store only a per-tree ``hasfriends`` flag.

    In a flagged tree, a daughter k of the root is paired with the incoming particle
    ``in`` (code 2^n_out or 2^(n_out+1)) when the tree lists the branch k|in: the
    t-channel line that connects k to that beam.  This reproduces the momenta of
    Whizard's own events in samples/bwbw.ref for all 16 flagged trees; unflagged trees
    list such branches too but carry no friend."""
    root = (1 << n_out) - 1
    out = np.zeros_like(np.asarray(d1, np.int32))
    for t in range(out.shape[0]):
        if not flags[t]:
            continue
        for k in (int(d1[t][root - 1]), int(d2[t][root - 1])):
            for inc in (1 << n_out, 1 << (n_out + 1)):
                code = k | inc
                if code <= out.shape[1] and has_children[t][code - 1]:
                    out[t][k - 1] = inc
    return out


def _values(line: str, conv=float) -> List:
    parts = line.split()
    return [conv(v) for v in parts[1:]]


def read_ref(path: str):
    """Returns (process, has_friends[int per channel], events)."""
    with open(path) as fh:
        lines = fh.read().splitlines()
    hdr = [int(lines[i].split()[1]) for i in range(6)]
    n_channels, n_in, n_out, n_trees, _n_groves, n_x = hdr
    n_prt = (1 << (n_in + n_out)) - 1
    n_prt_out = (1 << n_out) - 1
    pos = 6
    d1 = np.zeros((n_trees, n_prt), np.int32)
    d2 = np.zeros_like(d1)
    hc = np.zeros_like(d1)
    mid = np.zeros((n_trees, n_prt_out), np.int32)
    mm = np.zeros((n_trees, n_prt_out))
    mw = np.zeros((n_trees, n_prt_out))
    friends_flag = np.zeros(n_trees, np.int32)
    for t in range(n_trees):
        d1[t] = _values(lines[pos], int)[:n_prt]
        d2[t] = _values(lines[pos + 1], int)[:n_prt]
        hc[t] = _values(lines[pos + 2], int)[:n_prt]
        friends_flag[t] = _values(lines[pos + 3], int)[0]
        mid[t] = _values(lines[pos + 4], int)[:n_prt_out]
        mm[t] = _values(lines[pos + 5])[:n_prt_out]
        mw[t] = _values(lines[pos + 6])[:n_prt_out]
        pos += 7
    flv_m = np.array(_values(lines[pos])[: n_in + n_out])
    flv_w = np.array(_values(lines[pos + 1])[: n_in + n_out])
    pos += 2
    fr = friends_from_trees(n_out, d1, d2, hc, friends_flag)
    proc = Process(n_in, n_out, d1, d2, hc, fr, mid, mm, mw, flv_m, flv_w,
                   n_x=n_x, name=path.rsplit("/", 1)[-1], sqrts=0.0)
    n_lines = 5 + n_in + n_out
    body = [ln for ln in lines[pos:] if ln.strip()]
    n_ev = len(body) // n_lines
    ch = np.zeros(n_ev, np.int32)
    x = np.zeros((n_ev, n_x))
    pin = np.zeros((n_ev, n_in, 4))
    pout = np.zeros((n_ev, n_out, 4))
    vol = np.zeros(n_ev)
    ok = np.zeros(n_ev, np.int8)
    fac = np.zeros((n_ev, n_channels))
    for i in range(n_ev):
        blk = body[i * n_lines:(i + 1) * n_lines]
        ch[i] = int(blk[0].split()[1]) - 1
        x[i] = [float(v) for v in blk[1].split()[1:1 + n_x]]
        for k in range(n_in + n_out):
            v = [float(s) for s in blk[2 + k].split()[:4]]
            if k < n_in:
                pin[i, k] = v
            else:
                pout[i, k - n_in] = v
        vol[i] = float(blk[2 + n_in + n_out].split()[1])
        ok[i] = int(blk[3 + n_in + n_out].split()[1])
        fac[i] = [float(v) for v in blk[4 + n_in + n_out].split()[1:1 + n_channels]]
    return proc, friends_flag, RefEvents(ch, x, pin, pout, vol, ok, fac)
