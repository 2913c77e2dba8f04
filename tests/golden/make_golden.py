"""Generates the committed fixtures under tests/golden/.

  ac_lowpass_800hz_100khz_255.npy  the AC low-pass FIR the lambda stage uses
      (Hamming-windowed sinc, cutoff 800 Hz at 100 kHz, 255 taps, unit DC
      gain) -- the reference needs an AC filter for lambda output and ships
      none usable here (its equiripple designer is not reproduced).
  bm_cfg1_2ms.npz  FP32-oracle BM velocity / stats of config 1 (1 kHz,
      60 dB SPL) cut to a 2 ms block, pinning the oracle across changes.

Run: python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from cochlearmodel_gb300 import ihc, model  # noqa: E402
from oracle import oracle as orc  # noqa: E402
from tests import cases  # noqa: E402


def main():
    np.save(os.path.join(HERE, "ac_lowpass_800hz_100khz_255.npy"), ihc.design_ac_lowpass())
    mv = model.ModelVectors.build()
    cfg, sc, gamma, units, x, rows = cases.cfg1_slice(mv, ms=2.0)
    v, failed, st = orc.bm_run(mv.section_params(), gamma, sc, units, x, rows, threads=1)
    e = int(units["end"][0])
    np.savez_compressed(os.path.join(HERE, "bm_cfg1_2ms.npz"), v=v[:e], failed=failed[:e],
                        substeps=st["substeps"], iterations=st["iterations"],
                        sweeps=st["sweeps"])


if __name__ == "__main__":
    main()
