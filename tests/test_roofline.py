"""The byte model of the roofline (CPU): per-phase per-particle figures of
the compulsory-traffic model and the whole-step total."""
from mrsph import roofline


def test_per_particle_figures_3d_fp32():
    pp = roofline.per_particle_bytes(3, "fp32")
    assert roofline.total_bytes_per_particle(3, "fp32") == 344
    assert pp["density"] == 28 and pp["force1"] == 56 and pp["force2"] == 72


def test_whole_step_bytes():
    n, ls, cells = 1000, 50, 4000
    total = roofline.algorithmic_bytes(3, "fp32", n, ls, cells)
    assert total == 344 * n + 20 * ls + 8 * cells
    per_phase = roofline.step_bytes(3, "fp32", n, cells)
    assert sum(per_phase.values()) + 20 * ls == total
    assert roofline.algorithmic_bytes(3, "fp64", n, ls) == roofline.total_bytes_per_particle(3, "fp64") * n + 40 * ls
