"""Seeded input recipes for the reference-output fixtures.

Each recipe returns (marker, mask) as square uint8 arrays whose side is a
multiple of 512 -- the only inputs the reference's CUDA path accepts
(4-connectivity, uint8, square, IWPP MP DQ/src/MorphologicalReconstruction.cu:1245).
The generator is bit-identical on every host, so a fixture only records the
recipe name and the SHA-256 of the reference's output.
"""
from iwpp import synth


def uniform_512():
    # the reference's own generator law (testCaseGenerator.cu:28-35), its seed 1312
    return synth.uniform_pair(512, 512, 1312)


def hdome_512_h20():
    mask = synth.noise_mask(512, 512, synth.U8, 11, 4.0, 30)
    return synth.hdome_marker(mask, 20), mask


def cfg0_4conn_h40():
    return synth.config0()


def sparse_1024():
    mask = synth.noise_mask(1024, 1024, synth.U8, 12, 6.0, 50)
    return synth.sparse_marker(mask, 12, 0.001), mask


def hdome_2048_h100():
    mask = synth.noise_mask(2048, 2048, synth.U8, 13, 8.0, 500)
    return synth.hdome_marker(mask, 100), mask


def spiral_1024():
    marker, mask, _ = synth.spiral_case(1024, 1024, synth.U8, seed=14, sigma=8.0, arm_pitch=64, nseeds=8)
    return marker, mask


def unclipped_512():
    # marker not below the mask: the reference's caller clips first
    noise, _ = synth.uniform_pair(512, 512, 77)
    mask = synth.noise_mask(512, 512, synth.U8, 15, 3.0, 10)
    return noise, mask


def cfg1_h10():
    return synth.config1(10)


def cfg1_h40():
    return synth.config1(40)


def cfg1_h100():
    return synth.config1(100)


RECIPES = {f.__name__: f for f in (uniform_512, hdome_512_h20, cfg0_4conn_h40, sparse_1024, hdome_2048_h100,
                                    spiral_1024, unclipped_512, cfg1_h10, cfg1_h40, cfg1_h100)}
