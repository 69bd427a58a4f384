"""Generate the per-step digests of the parity configurations from the CPU
oracle (numpy stencils, SciPy SuperLU for the Stokes solve), for the GPU
trajectory tests in tests/test_gpu_configs.py.

  box100_weno5_100steps.npz
                    100 x 100, WENO5, 100 time steps (3 Picard sweeps each):
                    per step dt, the sweeps' residual norms and a digest of
                    every field of tests/configs.py DIGEST_FIELDS; the full
                    fields x, W, U, P after steps 1 and 10
  box400_<s>_3steps.npz
                    400 x 400, s = weno5 or quick, 3 time steps, same content
                    (one 400^2 sparse-LU solve takes about 100 s here)

The initial conditions and the white-noise draws are regenerated from their
seeds (tests/configs.py) by whoever reads the files; each file keeps a
checksum of the draws it used.  Run from the repository root:

    python tests/golden/make_configs.py [box100] [box400_weno5] [box400_quick]
"""
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path[:0] = [ROOT, os.path.join(ROOT, "oracle"), os.path.join(ROOT, "tests")]
import xcore_oracle as O  # noqa: E402
import configs as C  # noqa: E402


def run(cfg, scheme, steps, full_at, out_name):
    par, g, sc, ns, x0, draws, (re0, rs0) = C.setup(cfg, scheme=scheme)
    st = O.initialize(g, par, sc, ns, x0, re0, rs0)
    dt = sc["dt0"]
    out = {"x0_digest": C.digest(x0), "draw_checksum": np.array([float((re0 * re0).sum() + rs0.sum())])}
    dts, norms, dig = [], [], []
    t0 = time.time()
    for step in range(1, steps + 1):
        re, rs = draws.next()
        out["draw_checksum"] = out["draw_checksum"] + float((re * re).sum() + rs.sum())
        dt_used = dt
        dt, nrm = O.timestep(st, g, par, sc, ns, step, dt, re, rs, sweeps=3)
        dts.append(dt_used)
        norms.append([n[0] for n in nrm])
        dig.append(np.stack([C.digest(getattr(st, f)) for f in C.DIGEST_FIELDS]))
        if step in full_at:
            for f in ("x", "W", "U", "P"):
                out[f"s{step}_{f}"] = getattr(st, f).copy()
        print(f"{out_name}: step {step} dt {dt_used:.6e} resnorm {norms[-1][-1]:.3e} "
              f"({time.time() - t0:.0f} s)", flush=True)
    out["dt"] = np.array(dts)
    out["dt_next"] = np.array([dt])
    out["resnorm"] = np.array(norms)
    out["digest"] = np.stack(dig)
    out["fields"] = np.array(C.DIGEST_FIELDS)
    np.savez_compressed(os.path.join(HERE, out_name), **out)


if __name__ == "__main__":
    which = sys.argv[1:] or ["box100", "box400_weno5", "box400_quick"]
    if "box100" in which:
        run("box100", "weno5", 100, (1, 10), "box100_weno5_100steps.npz")
    for s in ("weno5", "quick"):
        if f"box400_{s}" in which:
            run("box400", s, 3, (), f"box400_{s}_3steps.npz")
