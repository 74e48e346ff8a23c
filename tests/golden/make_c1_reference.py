"""Generates tests/golden/c1_reference_16k.npz: the procedural Cornell box (256x256, depth 4)
rendered by the CPU oracle with 16,384 samples per pixel, every path's radiance summed in
double precision. It is the converged image the GPU renders' RMSE is stated against.

The samples are [2^20, 2^20 + 16384), disjoint from the ones a test render uses, so the
reference's own noise is independent of the image it judges. About 8 minutes on 8 cores:

    python tests/golden/make_c1_reference.py
"""
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

import lavaframe_gb300 as lf  # noqa: E402
import oracle  # noqa: E402

FIRST = 1 << 20
SPP = 16384
CHUNK = 64


def main():
    from lavaframe_gb300 import build

    build.build_core()
    build.build_oracle()
    s = lf.HostScene().gen_cornell(256, 256).build()
    p = s.render_params()
    total = np.zeros((p.height, p.width, 3), np.float64)
    t0 = time.time()
    for k in range(0, SPP, CHUNK):
        _, paths, _ = oracle.render(s.view(), p, FIRST + k, CHUNK, want_paths=True)
        total += paths.astype(np.float64).sum(axis=0)
        if k % 2048 == 0:
            print(f"{k + CHUNK} spp, {time.time() - t0:.0f} s", flush=True)
    mean = total / SPP
    np.savez_compressed(ROOT / "tests" / "golden" / "c1_reference_16k.npz", mean=mean.astype(np.float32),
                        first_sample=FIRST, spp=SPP)
    print("mean radiance", float(mean.mean()))


if __name__ == "__main__":
    main()
