"""Reader for MuMFiM's fiber-network text format and its ``.params`` file.

Network file (src/mumfim/microscale/FiberNetworkIO.cc:47-97)::

    n_nodes n_fibers n_periodic
    x y z                     (n_nodes lines)
    n0 n1                     (n_fibers lines, 0-based node ids)
    a b                       (n_periodic lines, 1-based; read and ignored here)

Params file (src/mumfim/microscale/FiberNetworkIO_impl.h:17-58)::

    n_reactions n_fibers
    0 radius E density                    (linear reaction)
    1 radius E B length_ratio_trns density  (nonlinear reaction)
    reaction_id                           (n_fibers lines)

Tokens are whitespace separated, as ``operator>>`` reads them. Fiber area is
``radius * radius * pi`` (FiberNetworkIO_impl.h:26), formed by the solver.
"""
from __future__ import annotations

from dataclasses import dataclass, field
from typing import List

import numpy as np

LINEAR = 0
NONLINEAR = 1


@dataclass
class Reaction:
    """One fiber reaction (FiberReactions.h:15-43)."""

    law: int
    radius: float
    youngs_modulus: float
    density: float
    B: float = 0.0
    length_ratio_trns: float = 0.0


@dataclass
class FiberNetwork:
    """Nodes, fibers and reactions of one RVE network."""

    coords: np.ndarray  # (n_nodes, 3) float64
    connectivity: np.ndarray  # (n_fibers, 2) int32
    reactions: List[Reaction] = field(default_factory=list)
    fiber_reaction: np.ndarray | None = None  # (n_fibers,) int32
    scale_factor: float = 1.0

    @property
    def n_nodes(self) -> int:
        return int(self.coords.shape[0])

    @property
    def n_fibers(self) -> int:
        return int(self.connectivity.shape[0])

    def reaction0(self) -> Reaction:
        """The reaction the batched solve uses for every fiber
        (BatchedFiberRVEAnalysisExplicit.h:202-212)."""
        return self.reactions[0]


class NetworkFormatError(ValueError):
    pass


def _tokens(text: str) -> List[str]:
    return text.split()


def parse_network(text: str) -> tuple[np.ndarray, np.ndarray]:
    tok = _tokens(text)
    if len(tok) < 3:
        raise NetworkFormatError("network header needs 'n_nodes n_fibers n_periodic'")
    nn, ne, npd = int(tok[0]), int(tok[1]), int(tok[2])
    if nn < 0 or ne < 0 or npd < 0:
        raise NetworkFormatError("negative counts in the network header")
    need = 3 + 3 * nn + 2 * ne + 2 * npd
    if len(tok) < need:
        raise NetworkFormatError(f"network file truncated: {len(tok)} tokens, {need} needed")
    p = 3
    coords = np.array(tok[p:p + 3 * nn], dtype=np.float64).reshape(nn, 3)
    p += 3 * nn
    conn = np.array([int(t) for t in tok[p:p + 2 * ne]], dtype=np.int64).reshape(ne, 2)
    if ne and (conn.min() < 0 or conn.max() >= nn):
        # FiberNetworkIO.cc:87-89 notes 1-based files as the usual culprit.
        raise NetworkFormatError("fiber references a node id outside [0, n_nodes)")
    return coords, conn.astype(np.int32)


def parse_params(text: str, n_fibers: int) -> tuple[List[Reaction], np.ndarray]:
    tok = _tokens(text)
    if len(tok) < 2:
        raise NetworkFormatError("params header needs 'n_reactions n_fibers'")
    nr, ne = int(tok[0]), int(tok[1])
    if ne != n_fibers:
        # FiberNetworkIO_impl.h:71-74 asserts the same
        raise NetworkFormatError(
            f"params file lists {ne} fibers, the network has {n_fibers}")
    p = 2
    reactions: List[Reaction] = []
    for _ in range(nr):
        law = int(tok[p]); p += 1
        if law == LINEAR:
            r, E, rho = (float(t) for t in tok[p:p + 3]); p += 3
            reactions.append(Reaction(LINEAR, r, E, rho))
        elif law == NONLINEAR:
            r, E, B, lt, rho = (float(t) for t in tok[p:p + 5]); p += 5
            reactions.append(Reaction(NONLINEAR, r, E, rho, B, lt))
        else:
            raise NetworkFormatError(f"unknown reaction type {law}")
    if len(tok) < p + ne:
        raise NetworkFormatError("params file truncated in the per-fiber reaction list")
    fr = np.array([int(t) for t in tok[p:p + ne]], dtype=np.int32)
    if ne and (fr.min() < 0 or fr.max() >= max(nr, 1)):
        raise NetworkFormatError("fiber reaction id out of range")
    return reactions, fr


def load_network(path: str, params_path: str | None = None) -> FiberNetwork:
    """FiberNetworkLibrary::load(net, net + ".params") (FiberNetworkLibrary.cc:17-60)."""
    with open(path, "r") as fh:
        coords, conn = parse_network(fh.read())
    with open(params_path or path + ".params", "r") as fh:
        reactions, fr = parse_params(fh.read(), conn.shape[0])
    return FiberNetwork(coords, conn, reactions, fr)


def format_network(net: FiberNetwork) -> str:
    lines = [f"{net.n_nodes} {net.n_fibers} 0"]
    lines += [f"{x:.17g} {y:.17g} {z:.17g}" for x, y, z in net.coords]
    lines += [f"{a} {b}" for a, b in net.connectivity]
    return "\n".join(lines) + "\n"


def format_params(net: FiberNetwork) -> str:
    lines = [f"{len(net.reactions)} {net.n_fibers}"]
    for r in net.reactions:
        if r.law == LINEAR:
            lines.append(f"0 {r.radius:.17g} {r.youngs_modulus:.17g} {r.density:.17g}")
        else:
            lines.append(f"1 {r.radius:.17g} {r.youngs_modulus:.17g} {r.B:.17g} "
                         f"{r.length_ratio_trns:.17g} {r.density:.17g}")
    fr = net.fiber_reaction if net.fiber_reaction is not None else np.zeros(net.n_fibers, np.int32)
    lines += [str(int(i)) for i in fr]
    return "\n".join(lines) + "\n"
