"""Generate the golden fixtures of this folder from the independent pure-Python
restatement (pyref.py).  Run from the repository root:  python tests/golden/make_golden.py

Each fixture holds the input mask, tau, the number of steps, the final populations
(the buffer the next step reads), the final macro texels (ux, uy, rho, w) and the final
info records.  Sizes are kept to a few thousand cells so that pure Python finishes in
seconds.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
import pyref  # noqa: E402

CASES = [
    # name, scene, nx, ny, tau, lid/inlet, steps, edit
    ("cavity_12x10", "cavity", 12, 10, 0.6, 0.1, 6, None),
    ("custom_10x8", "custom", 10, 8, 0.56, None, 5, "force"),
    ("poiseuille_64x60", "poiseuille", 64, 60, 0.56, 0.12, 3, None),
    ("cavity_obstacle_64x64", "cavity", 64, 64, 0.6, 0.1, 4, "obstacle"),
]


def run(name, scene, nx, ny, tau, speed, steps, edit):
    kw = {}
    if scene == "cavity" and speed is not None:
        kw["lid"] = speed
    if scene == "poiseuille" and speed is not None:
        kw["inlet"] = speed
    info0 = pyref.mask(nx, ny, scene, **kw)
    sim = pyref.PyRef(info0, tau, 1 if scene == "cavity" else 0)
    if edit == "force":
        # three force cells written after initialisation (as a force stroke is) with a
        # short countdown: they turn into bulk cells mid-run
        for x, bi in ((3, 2), (4, 3), (5, 9)):
            sim.info[3, x] = (6, bi, 0.05, -0.03)
    info_init = sim.info.copy()
    host_info = info0.copy()
    for s in range(steps):
        if edit == "obstacle" and s == 2:
            sim.add_obstacle(host_info, 32, 30)
        sim.step()
    np.savez_compressed(os.path.join(HERE, name + ".npz"), info_in=info0, info_init=info_init, tau=np.float32(tau),
                        steps=np.int32(steps), scene=np.array(scene), edit=np.array(edit or ""),
                        speed=np.float32(speed if speed is not None else 0.0),
                        pops=sim.A, macro=sim.macro, info_out=sim.info)
    print(name, "done")


if __name__ == "__main__":
    for case in CASES:
        run(*case)
