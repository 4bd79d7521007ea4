"""Writes pna_molecule.json: the p-nitroaniline molecule of the reference's
tests (tests/dump_pyscf.py, the `pna_xyz` block, from which the reference's
tests/pna.hdf5 was made with PySCF), as atomic numbers and positions in bohr.

The reference's functional tests (tests/test_functionality.py,
tests/test_solver.py, tests/test_gradients.py) read the molecule from
pna.hdf5 (h5py, PySCF's Angstrom-to-bohr conversion); this script reads the
same coordinates from dump_pyscf.py as text and converts them with PySCF's
constant (1 bohr = 0.52917721092 Angstrom).  Run where the reference is
mounted:

    python tests/golden/make_pna_molecule.py
"""
import json
import os
import re

HERE = os.path.dirname(os.path.abspath(__file__))
REF = os.environ.get("CPPE_REFERENCE_DIR", "/root/reference")
BOHR_ANGSTROM = 0.52917721092
Z = {"H": 1, "C": 6, "N": 7, "O": 8}


def main():
    with open(os.path.join(REF, "tests", "dump_pyscf.py")) as f:
        text = f.read()
    block = re.search(r'pna_xyz\s*=\s*"""(.*?)"""', text, re.S).group(1)
    atoms = [line.split() for line in block.strip().splitlines()]
    out = {"source": "reference tests/dump_pyscf.py (pna_xyz), Angstrom / 0.52917721092",
           "Z": [Z[a[0]] for a in atoms],
           "xyz_bohr": [[float(c) / BOHR_ANGSTROM for c in a[1:4]] for a in atoms]}
    with open(os.path.join(HERE, "pna_molecule.json"), "w") as f:
        json.dump(out, f, indent=1)
    print(len(atoms), "atoms")


if __name__ == "__main__":
    main()
