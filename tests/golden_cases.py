"""The fixed query sets behind the committed golden fixtures (tests/golden/*.npz)."""
import numpy as np

from pltfalcor_gb300 import workloads as W


def cases(profiles):
    rd = W.rough_dielectric_batch(n=65536, profiles=profiles).subset(np.arange(256))
    mm = W.mixed_material_batch(n=8 * 4096, profiles=profiles)
    mm1 = mm.subset(np.arange(1024))
    mm4 = W.mixed_material_batch(n=8 * 512, profiles=profiles, hwss=4).subset(np.arange(512))
    return {"rough_dielectric_256": rd, "mixed_material_1024": mm1, "mixed_material_hwss4_512": mm4}
