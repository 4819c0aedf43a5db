"""The oracle's optional threads (used only to time a multi-core CPU beside
the single-core reference arm): in red-black order the sweeps give the same
fields on any number of threads, and the norm differs only by its sum's
order."""
import numpy as np

from oracle import oracle as orc
from stroemung_gb300 import presets


def _run(threads):
    rects = presets.random_rectangles(256, 64, 6, 3, x_margin=16)
    g = presets.channel(256, 64, rects)
    o = orc.OracleSim(kind=g["kind"], wall_uv=g["wall_uv"], u=g["u"], v=g["v"], p=g["p"],
                      dx=0.04, dy=0.04, delt=0.01, gamma=0.9, reynolds=300.0, eps=1e-3,
                      omega=1.7, max_iterations=60, tau=0.5, sor_order=orc.RED_BLACK)
    o.set_threads(threads)
    res = [o.tick() for _ in range(3)]
    return res, {n: o.field(n) for n in ("u", "v", "p")}


def test_threads_change_only_the_norms_summation_order():
    orc.build()
    r1, f1 = _run(1)
    r4, f4 = _run(4)
    for (i1, n1), (i4, n4) in zip(r1, r4):
        assert i1 == i4
        assert abs(n1 - n4) <= 1e-12 * abs(n1)
    for n in f1:
        assert np.array_equal(f1[n], f4[n]), n
