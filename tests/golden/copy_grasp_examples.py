"""Copies the GRASP-written example data the tests read into
tests/golden/grasp_examples/. Run from the repository root, where the
reference tree is present:

    python tests/golden/copy_grasp_examples.py /root/reference

The files come from src/appl/rhfszeeman95/examples of the reference. They
are outputs of GRASP runs, copied byte for byte:

data_He/3Pn6  He, 2 electrons, 472 CSFs in three J blocks of odd parity
              (point nucleus, 220-point grid, c = 137.0359895):
              .c CSF list, .w orbitals (rmcdhf), .sum rmcdhf summary
              (Dirac-Coulomb energies), .cm / .csum rci mixing file and
              summary (with the transverse photon interaction).
data_Ge/2Fn5  Ge II, 31 electrons, 1850 CSFs in two blocks (J = 5/2-, 7/2-;
              Fermi nucleus, 590-point grid): .c, .w, .m (rmcdhf mixing,
              Dirac-Coulomb), .sum, .cm, .csum, isodata.

The tests use them to pin the oracle and the GPU path on data GRASP
produced: grid, quadrature and moments of GRASP's orbitals, the R^k and
I(ab) tables on those orbitals, the file readers and writers byte for byte,
and the rmcdhf Dirac-Coulomb energies of the CSF lists.
"""
import os
import shutil
import sys

FILES = {
    "data_He": ["3Pn6.c", "3Pn6.w", "3Pn6.sum", "3Pn6.cm", "3Pn6.csum", "isodata"],
    "data_Ge": ["2Fn5.c", "2Fn5.w", "2Fn5.m", "2Fn5.sum", "2Fn5.cm", "2Fn5.csum", "isodata"],
}


def main(ref_root):
    src_root = os.path.join(ref_root, "src", "appl", "rhfszeeman95", "examples")
    dst_root = os.path.join(os.path.dirname(os.path.abspath(__file__)), "grasp_examples")
    for d, names in FILES.items():
        os.makedirs(os.path.join(dst_root, d), exist_ok=True)
        for n in names:
            shutil.copyfile(os.path.join(src_root, d, n), os.path.join(dst_root, d, n))
            print(os.path.join(d, n))


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
