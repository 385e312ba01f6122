"""Copy the reference's regression-test inputs and stored logs used as
golden fixtures (run in a checkout that has the reference next to it).

The files are the reference's own data: eight configurations of its
`standard_2d` program (Cartesian and axisymmetric with the standard
two-reaction chemistry, Cartesian with three-mode Helmholtz
photoionization, and the air chemistry file with 8 species and 25 reactions
axisymmetric and Cartesian with photoionization and axisymmetric with
both, twice axisymmetric with six mobile ion species, and a grounded rod
electrode in the Cartesian domain under a positive and a negative applied
field, without and with photoionization), the transport and
reaction data they read, and the regression logs its test runner compares
at rtol 1e-5 (programs/standard_2d/tests/, tools/compare_logs.py); and the
3D configurations of its `standard_3d` program: the standard chemistry,
the small air chemistry (electron-temperature rates, ignored species) and
the same with photoionization (programs/standard_3d/tests/).
"""
import os
import shutil
import sys

SRC = "programs/standard_2d/tests"
FILES = ["test_2d.cfg", "test_2d_rtest.log", "test_cyl.cfg", "test_cyl_rtest.log",
         "test_2d_photoi.cfg", "test_2d_photoi_rtest.log", "td_air_siglo_swarm.txt",
         "test_cyl_chem.cfg", "test_cyl_chem_rtest.log", "test_2d_photoi_chem.cfg",
         "test_2d_photoi_chem_rtest.log", "air_chemistry_v1.txt", "test_cyl_ion_motion.cfg",
         "test_cyl_ion_motion_rtest.log", "test_cyl_ion_motion_v2.cfg", "test_cyl_ion_motion_v2_rtest.log",
         "test_cyl_photoi_chem.cfg", "test_cyl_photoi_chem_rtest.log",
         "test_2d_pos_electrode.cfg", "test_2d_pos_electrode_rtest.log",
         "test_2d_neg_electrode.cfg", "test_2d_neg_electrode_rtest.log",
         "test_2d_pos_electrode_photoi.cfg", "test_2d_pos_electrode_photoi_rtest.log",
         "test_2d_neg_electrode_photoi.cfg", "test_2d_neg_electrode_photoi_rtest.log"]


SRC_3D = "programs/standard_3d/tests"
FILES_3D = ["test_3d.cfg", "test_3d_rtest.log", "td_air_siglo_swarm.txt", "test_3d_chem.cfg",
            "test_3d_chem_rtest.log", "test_3d_photoi_chem.cfg", "test_3d_photoi_chem_rtest.log",
            "air_chemistry_small_v1.txt"]


def main(reference_root):
    here = os.path.dirname(os.path.abspath(__file__))
    for src, files, sub in ((SRC, FILES, "standard_2d"), (SRC_3D, FILES_3D, "standard_3d")):
        out = os.path.join(here, sub)
        os.makedirs(out, exist_ok=True)
        for f in files:
            shutil.copyfile(os.path.join(reference_root, src, f), os.path.join(out, f))
            print("copied", sub, f)


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
