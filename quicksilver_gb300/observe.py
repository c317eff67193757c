"""Observability outputs of a run: cumulative balance, fluence, census energy
spectrum and the CORAL2 correctness checks.

* ``cumulative_balance`` -- Tallies::_balanceCumulative (Tallies.cc:65), the
  sum of every finished cycle's 13 counters;
* fluence -- Fluence::compute (Tallies.cc:100-118), kept on the device by
  qsg_set_observers(QSG_OBSERVE_FLUENCE);
* energy spectrum -- EnergySpectrum::UpdateSpectrum / PrintSpectrum
  (EnergySpectrum.cc:12-59), kept on the device by
  qsg_set_observers(QSG_OBSERVE_SPECTRUM), written as ``<stem>.dat`` with one
  ``index<TAB>lower edge<TAB>count`` line per group edge;
* ``coral_benchmark_correctness`` -- the four checks of CoralBenchmark.cc:17-228
  with the reference's tolerances and messages.
"""
from __future__ import annotations

import sys

import numpy as np

from . import _native as N

B = N.BAL

# CoralBenchmark.cc:60-79: expected absorption / fission / scatter proportions
# of the two CORAL2 problems and the tolerance (percent) on their ratios
CORAL_RATIOS = {1: (0.04, 0.05, 1.0, 1.0), 2: (0.094, 0.075, 0.830, 1.1)}


def cumulative_balance(history_balance: np.ndarray) -> dict:
    """Sum of per-cycle counters ([cycles, 13]) as a name -> int dict."""
    tot = np.asarray(history_balance, dtype=np.uint64).reshape(-1, 13).sum(axis=0, dtype=np.uint64)
    return {name: int(tot[i]) for name, i in B.items()}


def _c_div(a, b) -> np.float64:
    """a / b as C evaluates it in double (x/0 = +-inf, 0/0 = nan)."""
    with np.errstate(divide="ignore", invalid="ignore"):
        return np.float64(a) / np.float64(b)


def balance_ratio_test(bal: dict, coral_benchmark: int):
    """BalanceRatioTest (CoralBenchmark.cc:46-118): the six relative ratios in
    C double arithmetic (a zero count gives inf, or nan, which passes, as
    there) and the reference's lines."""
    if coral_benchmark not in CORAL_RATIOS:
        raise ValueError(f"coralBenchmark must be 1 or 2, not {coral_benchmark}")
    absorb_r, fission_r, scatter_r, pct = CORAL_RATIOS[coral_benchmark]
    tol = pct / 100.0
    a, f, s = int(bal["absorb"]), int(bal["fission"]), int(bal["scatter"])
    with np.errstate(divide="ignore", invalid="ignore"):
        rel = {
            "Absorb to Scatter": abs(_c_div(a, absorb_r) * _c_div(scatter_r, s) - 1),
            "Absorb to Fission": abs(_c_div(a, absorb_r) * _c_div(fission_r, f) - 1),
            "Scatter to Absorb": abs(_c_div(s, scatter_r) * _c_div(absorb_r, a) - 1),
            "Scatter to Fission": abs(_c_div(s, scatter_r) * _c_div(fission_r, f) - 1),
            "Fission to Absorb": abs(_c_div(f, fission_r) * _c_div(absorb_r, a) - 1),
            "Fission to Scatter": abs(_c_div(f, fission_r) * _c_div(scatter_r, s) - 1),
        }
    ok = not any(v > tol for v in rel.values())
    if ok:
        msg = "PASS:: Absorption / Fission / Scatter Ratios maintained with %g%% tolerance" % (tol * 100.0)
    else:
        labels = {"Absorb to Scatter": "Absorb to Scatter:  ", "Absorb to Fission": "Absorb to Fission:  ",
                  "Scatter to Absorb": "Scatter to Absorb:  ", "Scatter to Fission": "Scatter to Fission: ",
                  "Fission to Absorb": "Fission to Absorb:  ", "Fission to Scatter": "Fission to Scatter: "}
        msg = "\n".join(["FAIL:: Absorption / Fission / Scatter Ratios NOT maintained with %g%% tolerance" %
                         (tol * 100.0),
                         "absorb:  %12d\t%g" % (a, absorb_r), "scatter: %12d\t%g" % (s, scatter_r),
                         "fission: %12d\t%g" % (f, fission_r)] +
                        ["Relative %s%g < %g" % (labels[k], v, tol) for k, v in rel.items()])
    return ok, msg, rel


def balance_event_test(bal: dict):
    """BalanceEventTest (CoralBenchmark.cc:120-152): facet crossings
    (segments - census - collisions, as uint64) within 1% of the collisions."""
    facet = (int(bal["num_segments"]) - int(bal["census"]) - int(bal["collision"])) % (1 << 64)
    ratio = abs(_c_div(facet, int(bal["collision"])) - 1)
    tolerance = 1.0
    ok = not (ratio > tolerance / 100.0)
    msg = ("PASS:: Collision to Facet Crossing Ratio maintained even balanced within %g%% tolerance" % tolerance
           if ok else
           " FAIL:: Collision to Facet Crossing Ratio balanced NOT maintained within %g%% tolerance\n"
           "\tFacet Crossing: %d\tCollision: %d\tRatio: %g" % (tolerance, facet, int(bal["collision"]), ratio))
    return ok, msg, ratio


def missing_particle_test(bal: dict):
    """MissingParticleTest (CoralBenchmark.cc:154-175): start + source +
    produce + split == absorb + census + escape + rr + fission."""
    gains = bal["start"] + bal["source"] + bal["produce"] + bal["split"]
    losses = bal["absorb"] + bal["census"] + bal["escape"] + bal["rr"] + bal["fission"]
    ok = gains == losses
    msg = ("PASS:: No Particles Lost During Run" if ok else
           "FAIL:: Particles Were Lost During Run, test for done should have failed")
    return ok, msg, (gains, losses)


def fluence_test(fluence: np.ndarray):
    """FluenceTest (CoralBenchmark.cc:177-228): max over cells of
    |cell - mean| / ((cell + mean) / 2) in percent, within 6%, evaluated as
    there: the mean from a running sum, the maximum by `max > d ? max : d`
    (a nan difference replaces the running maximum)."""
    f = np.asarray(fluence, dtype=np.float64)
    local_sum = float(np.cumsum(f)[-1]) if len(f) else 0.0
    average = _c_div(local_sum, len(f))
    with np.errstate(divide="ignore", invalid="ignore"):
        diff = (np.where(f > average, f - average, average - f) / ((f + average) / 2.0)) * 100
    max_diff = 0.0
    for d in diff.tolist():
        max_diff = max_diff if max_diff > d else d
    percent_tolerance = 6.0
    ok = not (max_diff > percent_tolerance)
    msg = ("PASS:: Fluence is homogenous across cells with %g%% tolerance" % percent_tolerance if ok else
           "FAIL:: Fluence not homogenous across cells within %g%% tolerance\n"
           "\tTry running more particles or more cycles to see if Max Percent Difference goes down.\n"
           "\tCurrent Max Percent Diff: %4.1f%%" % (percent_tolerance, max_diff))
    return ok, msg, max_diff


def coral_benchmark_correctness(bal: dict, fluence: np.ndarray, coral_benchmark: int, out=sys.stdout) -> dict:
    """coralBenchmarkCorrectness (CoralBenchmark.cc:17-44): prints the four
    checks and returns {name: passed}."""
    results = {}
    for name, header, (ok, msg, _) in (
            ("balance_ratio", "Testing Ratios for Absorbtion, Fission, and Scattering are maintained",
             balance_ratio_test(bal, coral_benchmark)),
            ("balance_event", "Testing balance between number of facet crossings and reactions",
             balance_event_test(bal)),
            ("missing_particle", "Test for lost / unaccounted for particles in this simulation",
             missing_particle_test(bal)),
            ("fluence", "Test Fluence for homogeneity across cells", fluence_test(fluence))):
        if out is not None:
            out.write(f"\n{header}\n{msg}\n")
        results[name] = ok
    return results


def write_energy_spectrum(stem: str, energies: np.ndarray, counts: np.ndarray) -> str:
    """PrintSpectrum (EnergySpectrum.cc:38-59): ``stem + ".dat"`` with
    ``index<TAB>energy edge<TAB>count`` for each of the G+1 entries."""
    path = stem + ".dat"
    with open(path, "w") as fh:
        for i, (e, c) in enumerate(zip(energies, counts)):
            fh.write(f"{i}\t{float(e):g}\t{int(c)}\n")
    return path


def cross_section_table(hp, material_names) -> str:
    """The file the reference writes when the deck sets crossSectionsOut
    (initMC.cc:392-490): per energy group its midpoint energy and, for every
    material in name order, the absorption, fission and scatter microscopic
    cross sections summed over the material's isotopes and their reactions,
    each divided by the isotope count (accumulated in the same order: isotope,
    reaction, group).  `material_names`: the materials in this problem's
    order, which is name order."""
    e = hp.array("energies")
    G = len(e) - 1
    iso_off = hp.array("isotope_reaction_offset")
    rtype = hp.array("reaction_type")
    xs = hp.array("reaction_xs").reshape(-1, G)
    mat_off = hp.array("material_isotope_offset")
    gid = hp.array("material_isotope_gid")
    kind = {N.QSG_REACT_ABSORPTION: 0, N.QSG_REACT_FISSION: 1, N.QSG_REACT_SCATTER: 2}
    table = []
    for m in range(len(material_names)):
        isos = gid[mat_off[m]:mat_off[m + 1]]
        acc = np.zeros((3, G))
        for iso in isos:
            for r in range(iso_off[iso], iso_off[iso + 1]):
                acc[kind[int(rtype[r])]] += xs[r] / float(len(isos))
        table.append(acc)
    order = sorted(range(len(material_names)), key=lambda m: material_names[m])
    energy = (e[:-1] + e[1:]) / 2.0
    lines = ["#group  energy" + "".join("  %s_a  %s_f  %s_s" % ((material_names[m],) * 3) for m in order)]
    for g in range(G):
        lines.append("%u  %g" % (g, energy[g]) +
                     "".join("  %g  %g  %g" % (table[m][0, g], table[m][1, g], table[m][2, g]) for m in order))
    return "\n".join(lines) + "\n"


def write_cross_sections(stem: str, hp, material_names) -> str:
    """Write cross_section_table to <stem>.dat, as the reference does; returns the path."""
    path = stem + ".dat"
    with open(path, "w") as f:
        f.write(cross_section_table(hp, material_names))
    return path
