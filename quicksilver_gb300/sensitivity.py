"""Derivatives of Quicksilver tallies with respect to cross-section scale
parameters, computed during tracking (differential-operator / likelihood-ratio
scores carried per history by the SENS instantiation of the tracking kernel).

A parameter ``Param(material, reaction, group_lo, group_hi, theta)`` multiplies
the microscopic cross sections of every reaction of type ``reaction``
(1 scatter, 2 absorption, 3 fission: NuclearDataReaction::Enum,
NuclearData.hh:33-40) of every isotope of ``material`` in groups
``[group_lo, group_hi)``.  The tables handed to the tracker are scaled by
theta (``scaled_problem``); the sensitivities are then d(tally)/d(theta) at
that theta.  Forward tracking is unchanged bit for bit: the balance counters
of a run with sensitivities are those of the same run without.

Tallies (accumulated over every cycle of a run):
  * ``flux_cell[c]``  group-summed track-length scalar flux of cell c
    (the reference's Tallies::TallyScalarFlux, Tallies.hh:350-354, summed over
    groups and cycles),
  * ``leak[p]``       weight escaping problem p through escape facets
    (MC_Facet_Crossing_Event.cc:23-70),
  * ``dflux[c, k]``, ``dleak[p, k]`` their derivatives in theta_k.

``tallies(theta, deck, params)`` exposes the run as a differentiable
function of a torch tensor theta (``torch.autograd.Function``): the forward
pass runs the GPU transport, the backward pass contracts the stored
derivatives with the incoming gradients.  torch is only imported when that
binding is used.
"""
from __future__ import annotations

from dataclasses import dataclass, replace

import numpy as np

from .monte_carlo import MonteCarlo
from .problem import Deck, HostProblem

SCATTER, ABSORPTION, FISSION = 1, 2, 3


@dataclass(frozen=True)
class Param:
    """theta scales reaction type `reaction` of `material` in groups
    [group_lo, group_hi), and every further (material, reaction, group_lo,
    group_hi) entry of `also` (one physical parameter tied across materials,
    e.g. the same parameter in every problem of a batch)."""
    material: int
    reaction: int
    group_lo: int
    group_hi: int
    theta: float = 1.0
    also: tuple = ()

    def entries(self) -> list:
        return [(self.material, self.reaction, self.group_lo, self.group_hi), *self.also]

    def shifted(self, material_offset: int) -> "Param":
        """The same parameter with every material index moved by an offset."""
        moved = [(m + material_offset, r, lo, hi) for (m, r, lo, hi) in self.entries()]
        return Param(*moved[0], theta=self.theta, also=tuple(moved[1:]))


def tie_across_problems(params, material_offsets) -> list:
    """Per-problem parameters (local material indices) tied across the
    problems of a batch whose materials start at material_offsets[p]."""
    out = []
    for prm in params:
        entries = [e for off in material_offsets[:-1] for e in prm.shifted(int(off)).entries()]
        out.append(Param(*entries[0], theta=prm.theta, also=tuple(entries[1:])))
    return out


def band_params(energies: np.ndarray, n_materials: int, reactions=(SCATTER, ABSORPTION),
                split_mev: float = 1.0) -> list:
    """One parameter per (material, reaction type, energy band); the bands
    split at the first group edge >= split_mev.  Order: material-major, then
    reaction, then band (low, high)."""
    energies = np.asarray(energies, dtype=np.float64)
    G = len(energies) - 1
    g1 = int(np.clip(np.searchsorted(energies, split_mev), 1, G - 1))
    out = []
    for m in range(n_materials):
        for r in reactions:
            out.append(Param(m, r, 0, g1))
            out.append(Param(m, r, g1, G))
    return out


def with_theta(params, theta) -> list:
    theta = np.asarray(theta, dtype=np.float64).reshape(-1)
    if len(theta) != len(params):
        raise ValueError(f"{len(theta)} theta values for {len(params)} parameters")
    return [replace(p, theta=float(t)) for p, t in zip(params, theta)]


def scaled_problem(deck: Deck, params) -> HostProblem:
    """The deck's tables with each parameter's cross sections multiplied by its theta."""
    hp = deck.build()
    for p in params:
        if p.theta != 1.0:
            for (m, r, lo, hi) in p.entries():
                hp.scale_xs(m, r, lo, hi, p.theta)
    return hp


def run_sensitivity(deck: Deck, params, n_steps: int | None = None, seed_offset: int = 0, **mc_options) -> dict:
    """Run the deck's cycles at the params' theta with sensitivity tallies.
    Returns flux_cell [C], dflux [C, K], leak [1], dleak [1, K], the cycle
    history and the segment count."""
    problem = scaled_problem(deck, params)
    mc = MonteCarlo(deck, problem=problem, seed_offset=seed_offset, **mc_options)
    try:
        mc.tracker.enable_sensitivity(params)
        hist = mc.run(n_steps)
        out = mc.tracker.read_sensitivity()
        out["history"] = hist
        out["segments"] = hist.segments()
        return out
    finally:
        mc.close()
        problem.close()


def _function():
    import torch

    class TallyFunction(torch.autograd.Function):
        """theta [K] -> (flux_cell [C], leak [1]); backward = J^T g with the
        Jacobian tallied by the sensitivity kernel in the same run."""

        @staticmethod
        def forward(ctx, theta, deck, params, n_steps, seed_offset, options):
            th = theta.detach().to("cpu", torch.float64).numpy()
            res = run_sensitivity(deck, with_theta(params, th), n_steps, seed_offset, **options)
            ctx.save_for_backward(torch.from_numpy(res["dflux"]), torch.from_numpy(res["dleak"]))
            ctx.theta_meta = (theta.dtype, theta.device)
            flux = torch.from_numpy(res["flux_cell"]).to(theta.device)
            leak = torch.from_numpy(res["leak"]).to(theta.device)
            return flux, leak

        @staticmethod
        def backward(ctx, g_flux, g_leak):
            dflux, dleak = ctx.saved_tensors
            dtype, device = ctx.theta_meta
            grad = torch.zeros(dflux.shape[1], dtype=torch.float64)
            if g_flux is not None:
                grad = grad + dflux.T @ g_flux.detach().to("cpu", torch.float64)
            if g_leak is not None:
                grad = grad + dleak.T @ g_leak.detach().to("cpu", torch.float64)
            return grad.to(device=device, dtype=dtype), None, None, None, None, None

    return TallyFunction


_TALLY_FUNCTION = None


def tallies(theta, deck: Deck, params, n_steps: int | None = None, seed_offset: int = 0, **options):
    """Differentiable (flux_cell, leak) of a whole run as a function of the
    torch tensor theta (one entry per parameter of `params`)."""
    global _TALLY_FUNCTION
    if _TALLY_FUNCTION is None:
        _TALLY_FUNCTION = _function()
    return _TALLY_FUNCTION.apply(theta, deck, list(params), n_steps, seed_offset, options)


def main(argv=None) -> None:
    """``python -m quicksilver_gb300.sensitivity DECK [--steps N] [--split-mev E]``:
    run the deck with one parameter per (material, {scatter, absorption},
    energy band) and print the total flux, the leakage and their derivatives."""
    import argparse
    import json
    ap = argparse.ArgumentParser(description=main.__doc__)
    ap.add_argument("deck")
    ap.add_argument("--steps", type=int, default=None, help="cycles (default: the deck's nSteps)")
    ap.add_argument("--split-mev", type=float, default=1.0)
    args = ap.parse_args(argv)
    deck = Deck.from_file(args.deck)
    hp = deck.build()
    params = band_params(hp.array("energies"), hp.num_materials, split_mev=args.split_mev)
    hp.close()
    res = run_sensitivity(deck, params, args.steps)
    print(json.dumps({"segments": res["segments"], "flux_total": float(res["flux_cell"].sum()),
                      "leak": float(res["leak"].sum()),
                      "dflux_total": res["dflux"].sum(axis=0).tolist(), "dleak": res["dleak"].sum(axis=0).tolist(),
                      "params": [[p.material, p.reaction, p.group_lo, p.group_hi] for p in params]}))


if __name__ == "__main__":
    main()


__all__ = ["Param", "SCATTER", "ABSORPTION", "FISSION", "band_params", "with_theta", "scaled_problem",
           "tie_across_problems", "run_sensitivity", "tallies"]
