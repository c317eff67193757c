"""Write the benchmark and test decks (Quicksilver input format) into this folder.

Run ``python -m quicksilver_gb300.decks.make_decks``.  Every random draw uses a
fixed numpy seed, so the decks are reproducible.  Benchmark workloads:

* ``config1.inp``  homogeneous 10^3-cell, 10 cm box, 1 material / 1 isotope,
  scatter 0.7 + absorption 0.3 of 1 barn (nReactions 3 with fission ratio 0,
  which gives [scatter, fission(0), absorption] -- with 2 reactions the
  reference makes scatter + fission, NuclearData.cc:136-183), 1e5 particles,
  10 cycles, dt 1e-8 s, 230 groups over [1e-9, 20] MeV, one domain.
* ``config2.inp``  40^3 cells over a 40 cm cube; 3 materials as a brick plus
  spheres of radius 16 and 8 cm about the centre (the last matching geometry
  wins, MC_Domain.cc:440-449); 2 isotopes and 3 reactions per material with
  totals drawn from U[0.5, 5] barn and scatter fractions from U[0.5, 0.95];
  polynomial-in-log10(E) cross sections with C ~ U[-0.02, 0.02],
  D ~ U[-0.5, 0.1]; 1e6 particles, 20 cycles.  numpy default_rng(7).
* ``config4.inp``  config-1 box and mesh with 3 materials (spheres of radius
  2 and 4 cm about the centre), escape boundaries, 1e6 particles, 20 cycles;
  numpy default_rng(4).
* ``config3()`` / ``config5()`` return deck strings (64 uneven problems; 8
  replicas of a 5-slab 64^3 problem) instead of writing files.

Test decks (small, seconds on one CPU core): limit cases mirroring the
reference's example physics (all-absorb, all-escape, no-collision,
scatter-only, fission with secondaries, octant boundaries, energy-dependent
cross sections, default problem).
"""
from __future__ import annotations

from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent


def simulation(**kw) -> str:
    base = dict(dt="1e-08", boundaryCondition="reflect", lx=10, ly=10, lz=10, nParticles=100000, nSteps=10,
                nx=10, ny=10, nz=10, seed=1029384756, xDom=1, yDom=1, zDom=1, eMax=20, eMin="1e-09",
                nGroups=230)
    base.update(kw)
    return "Simulation:\n" + "".join(f"   {k}: {v}\n" for k, v in base.items()) + "\n"


def brick(material: str, x0, x1, y0, y1, z0, z1) -> str:
    return (f"Geometry:\n   material: {material}\n   shape: brick\n   xMax: {x1}\n   xMin: {x0}\n"
            f"   yMax: {y1}\n   yMin: {y0}\n   zMax: {z1}\n   zMin: {z0}\n\n")


def sphere(material: str, r, cx, cy, cz) -> str:
    return (f"Geometry:\n   material: {material}\n   shape: sphere\n   radius: {r}\n   xCenter: {cx}\n"
            f"   yCenter: {cy}\n   zCenter: {cz}\n\n")


def material(name: str, *, total, scatter, absorb, fission=0, n_iso=1, n_react=3, source="1e+10",
             xs_s="flat", xs_a="flat", xs_f="flat", mass=None) -> str:
    lines = [f"   name: {name}", f"   nIsotopes: {n_iso}", f"   nReactions: {n_react}",
             f"   sourceRate: {source}", f"   totalCrossSection: {total}",
             f"   absorptionCrossSection: {xs_a}", f"   fissionCrossSection: {xs_f}",
             f"   scatteringCrossSection: {xs_s}", f"   absorptionCrossSectionRatio: {absorb}",
             f"   fissionCrossSectionRatio: {fission}", f"   scatteringCrossSectionRatio: {scatter}"]
    if mass is not None:
        lines.insert(1, f"   mass: {mass}")
    return "Material:\n" + "\n".join(lines) + "\n\n"


def cross_section(name: str, a=0, b=0, c=0, d=0, e=1, nu_bar=2.4) -> str:
    return (f"CrossSection:\n   name: {name}\n   A: {a}\n   B: {b}\n   C: {c}\n   D: {d}\n   E: {e}\n"
            f"   nuBar: {nu_bar}\n\n")


def drawn_materials(rng, names):
    """Materials with 2 isotopes, scatter + absorption, polynomial cross sections."""
    mats, xss = [], []
    for name in names:
        total = rng.uniform(0.5, 5.0)
        sfrac = rng.uniform(0.5, 0.95)
        cs, ds = rng.uniform(-0.02, 0.02), rng.uniform(-0.5, 0.1)
        ca, da = rng.uniform(-0.02, 0.02), rng.uniform(-0.5, 0.1)
        xss.append(cross_section(f"{name}_s", c=repr(float(cs)), d=repr(float(ds)), e=0))
        xss.append(cross_section(f"{name}_a", c=repr(float(ca)), d=repr(float(da)), e=0))
        mats.append(material(name, total=repr(float(total)), scatter=repr(float(sfrac)),
                             absorb=repr(float(1.0 - sfrac)), n_iso=2, xs_s=f"{name}_s", xs_a=f"{name}_a"))
    return "".join(mats) + "".join(xss) + cross_section("flat")


def config1() -> str:
    return (simulation() + brick("sourceMaterial", 0, 10, 0, 10, 0, 10) +
            material("sourceMaterial", total="1.0", scatter="0.7", absorb="0.3") + cross_section("flat"))


def config2() -> str:
    rng = np.random.default_rng(7)
    return (simulation(lx=40, ly=40, lz=40, nx=40, ny=40, nz=40, nParticles=1000000, nSteps=20, seed=7) +
            brick("matA", 0, 40, 0, 40, 0, 40) + sphere("matB", 16, 20, 20, 20) + sphere("matC", 8, 20, 20, 20) +
            drawn_materials(rng, ["matA", "matB", "matC"]))


def config4() -> str:
    rng = np.random.default_rng(4)
    return (simulation(boundaryCondition="escape", nParticles=1000000, nSteps=20) +
            brick("matA", 0, 10, 0, 10, 0, 10) + sphere("matB", 4, 5, 5, 5) + sphere("matC", 2, 5, 5, 5) +
            drawn_materials(rng, ["matA", "matB", "matC"]))


def config3(n_problems: int = 64, seed: int = 3) -> list:
    """The uneven ensemble tracked as one batch: mesh edge n drawn from
    {8, 16, 24, 32, 48} with 1-cm cells (lx = n), particle count log-uniform in
    [1e4, 2e6], 1-3 materials as nested spheres of radii 0.2n and 0.4n about the
    centre with config-2-style polynomial cross sections, 230 groups, 10
    cycles; problem p carries seed 3000 + p (numpy default_rng(seed))."""
    rng = np.random.default_rng(seed)
    decks = []
    for p in range(n_problems):
        n = int(rng.choice([8, 16, 24, 32, 48]))
        n_part = int(round(float(np.exp(rng.uniform(np.log(1e4), np.log(2e6))))))
        n_mat = int(rng.integers(1, 4))
        names = [f"m{p}_{k}" for k in range(n_mat)]
        c = n / 2
        geo = brick(names[0], 0, n, 0, n, 0, n)
        if n_mat >= 2:
            geo += sphere(names[1], repr(0.4 * n), c, c, c)
        if n_mat >= 3:
            geo += sphere(names[2], repr(0.2 * n), c, c, c)
        text = (simulation(lx=n, ly=n, lz=n, nx=n, ny=n, nz=n, nParticles=n_part, nSteps=10, seed=3000 + p) +
                geo + drawn_materials(rng, names))
        decks.append(text)
    return decks


def config5(n_replicas: int = 8, seed: int = 5, n_particles: int = 10_000_000) -> list:
    """The large batched + differentiated run: n_replicas copies of a 64^3-cell
    64 cm cube made of 5 slabs along z (thicknesses 64 x a Dirichlet(1,...,1)
    draw), 5 materials with config-2-style cross sections, 230 groups, escape
    boundaries, 1e7 particles, 20 cycles; replica r carries deck seed 5 + r
    (numpy default_rng(seed) draws the geometry and the materials once)."""
    rng = np.random.default_rng(seed)
    z = np.concatenate([[0.0], np.cumsum(rng.dirichlet(np.ones(5)) * 64.0)])
    z[-1] = 64.0
    names = [f"slab{k}" for k in range(5)]
    geo = "".join(brick(names[k], 0, 64, 0, 64, repr(float(z[k])), repr(float(z[k + 1]))) for k in range(5))
    mats = drawn_materials(rng, names)
    return [simulation(boundaryCondition="escape", lx=64, ly=64, lz=64, nx=64, ny=64, nz=64,
                       nParticles=n_particles, nSteps=20, seed=seed + r) + geo + mats
            for r in range(n_replicas)]


def small(**kw) -> str:
    sim = dict(lx=5, ly=5, lz=5, nx=5, ny=5, nz=5, nParticles=4000, nSteps=3, nGroups=16)
    sim.update(kw)
    return simulation(**sim)


def test_decks() -> dict:
    d = {}
    d["t_homog.inp"] = small() + brick("src", 0, 5, 0, 5, 0, 5) + material("src", total="1.0", scatter="0.7",
                                                                          absorb="0.3") + cross_section("flat")
    # every source particle is absorbed at its first collision (cf. reference AllAbsorb physics)
    d["t_absorb.inp"] = (small(dt="1e6", eMin="0.99999", eMax=1, nGroups=1, nSteps=2) +
                         brick("src", 0, 5, 0, 5, 0, 5) +
                         material("src", total="1e10", scatter=0, absorb=1, n_iso=3, n_react=9, source="1e-2") +
                         cross_section("flat"))
    # everything escapes (cf. AllEscape physics)
    d["t_escape.inp"] = (small(boundaryCondition="escape", nSteps=2) + brick("src", 0, 5, 0, 5, 0, 5) +
                         material("src", total="1e-20", scatter=1, absorb=0) + cross_section("flat"))
    # no collisions: everything censuses (cf. NoCollisions)
    d["t_nocoll.inp"] = (small(nSteps=2) + brick("src", 0, 5, 0, 5, 0, 5) +
                         material("src", total="1e-80", scatter=1, absorb=0) + cross_section("flat"))
    # scatter only, octant boundaries (escape on +x,+y,+z; reflect on -x,-y,-z)
    d["t_scatter_octant.inp"] = (small(boundaryCondition="octant", lx=20, ly=20, lz=20, nx=4, ny=4, nz=4) +
                                 brick("src", 0, 20, 0, 20, 0, 20) +
                                 material("src", total="0.198", scatter=1, absorb=0, n_iso=2) +
                                 cross_section("flat"))
    # fission producing secondaries: extra vault path (cf. CORAL2 physics)
    d["t_fission.inp"] = (small(nx=6, ny=6, nz=6, lx=6, ly=6, lz=6, dt="2e-09", lowWeightCutoff=0.001) +
                          brick("src", 0, 6, 0, 6, 0, 6) +
                          material("src", total="1.5", scatter=1, absorb="0.04", fission="0.3", n_iso=4,
                                   n_react=9, mass="12.011", xs_f="fis") +
                          cross_section("flat") + cross_section("fis", nu_bar=2.6))
    # energy-dependent cross sections and two materials (cf. NonFlatXC)
    rng = np.random.default_rng(11)
    d["t_nonflat.inp"] = (small(nx=6, ny=6, nz=6, lx=6, ly=6, lz=6, nGroups=40) + brick("matA", 0, 6, 0, 6, 0, 6) +
                          sphere("matB", 2, 3, 3, 3) + drawn_materials(rng, ["matA", "matB"]))
    # config-4 geometry in small: escape boundaries, 3 nested materials (sensitivity tests)
    rng = np.random.default_rng(5)
    d["t_sens.inp"] = (small(boundaryCondition="escape", nx=6, ny=6, nz=6, lx=6, ly=6, lz=6, nGroups=40) +
                       brick("matA", 0, 6, 0, 6, 0, 6) + sphere("matB", "2.4", 3, 3, 3) +
                       sphere("matC", "1.2", 3, 3, 3) + drawn_materials(rng, ["matA", "matB", "matC"]))
    # CORAL2-style problem 1 setup (the proportions CoralBenchmark.cc:60-65
    # expects: absorption 0.04, fission 0.05, scatter 1) with its checks on
    d["t_coral1.inp"] = (small(nx=6, ny=6, nz=6, lx=6, ly=6, lz=6, dt="2e-09", nParticles=8000, nSteps=5,
                               coralBenchmark=1) +
                         brick("src", 0, 6, 0, 6, 0, 6) +
                         material("src", total="1.5", scatter=1, absorb="0.04", fission="0.05", n_iso=4,
                                  n_react=9, mass="12.011") + cross_section("flat"))
    # no Geometry block: supplyDefaults problem (Parameters.cc:350-379)
    d["t_default.inp"] = small(nParticles=3000, nSteps=2, lx=10, ly=10, lz=10)
    return d


def main() -> None:
    (HERE / "config1.inp").write_text(config1())
    (HERE / "config2.inp").write_text(config2())
    (HERE / "config4.inp").write_text(config4())
    for name, text in test_decks().items():
        (HERE / name).write_text(text)


if __name__ == "__main__":
    main()
