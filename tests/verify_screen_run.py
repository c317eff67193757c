"""Whole device cycles of one deck through the screen-verification build of
the library (libqsg_verify.so), printed as one JSON line: the 13 balance
counters and the flux total of every cycle, and the device flag word.

Run by tests/test_gpu_verify_screen.py in a child process with
QSG_LIB=verify (the library variant is chosen when quicksilver_gb300._native
is first imported, so it cannot change within one process):

    QSG_LIB=verify python tests/verify_screen_run.py DECK.inp CYCLES [PARTICLES]
"""
import json
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT))

from quicksilver_gb300 import Deck, _native  # noqa: E402
from quicksilver_gb300.monte_carlo import MonteCarlo  # noqa: E402


def main() -> None:
    deck_path, cycles = Path(sys.argv[1]), int(sys.argv[2])
    overrides = {"nParticles": int(sys.argv[3])} if len(sys.argv) > 3 else None
    deck = Deck.from_file(deck_path, overrides)
    mc = MonteCarlo(deck)
    try:
        for _ in range(cycles):
            mc.cycle_init()
            mc.cycle_tracking()
            mc.cycle_finalize()
        hist = mc.history(0, cycles)
        flags = mc.device_status()
    finally:
        mc.close()
    print(json.dumps({"library": str(_native.LIB_PATH.name), "balance": hist.balance.tolist(),
                      "flux_total": hist.flux_total.tolist(), "flags": int(flags)}))


if __name__ == "__main__":
    main()
