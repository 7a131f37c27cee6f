"""The scene generators built into the small host-only library of the
oracle build (what the benchmark's reference arm uses) give, bit for bit,
the scenes of libfcdem.so's build of the same source."""
import numpy as np


def test_generator_builds_agree():
    from fullc0ntact_gb300 import _native, scenes
    from oracle import oracle as O
    try:
        a = scenes.packed_scene(20_000, grid=64)
        b = scenes.lattice_scene(3000)
        c = scenes.batch_scene(5000, seed=3)
        scenes.use_generator(O.scenegen())
        a2 = scenes.packed_scene(20_000, grid=64)
        b2 = scenes.lattice_scene(3000)
        c2 = scenes.batch_scene(5000, seed=3)
    finally:
        scenes.use_generator(_native.lib)
    for x, y in ((a, a2), (b, b2), (c, c2)):
        np.testing.assert_array_equal(x["pos"].view(np.uint32), y["pos"].view(np.uint32))
        np.testing.assert_array_equal(x["vel"].view(np.uint32), y["vel"].view(np.uint32))
