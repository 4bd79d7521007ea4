import gzip
import os
import shutil
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); parity tests of the kernels")


def golden(name):
    return os.path.join(GOLDEN, name)


@pytest.fixture(scope="session")
def golden_vectors():
    return dict(np.load(golden("ref_vectors.npz")))


@pytest.fixture(scope="session")
def unpacked(tmp_path_factory):
    """The gzipped potfiles unpacked into a temp dir (the reader takes paths)."""
    d = tmp_path_factory.mktemp("potfiles")
    out = {}
    for f in ("pna_6w.pot", "pna_6w_isopol.pot", "loprop_solvated_20.pot"):
        dst = os.path.join(d, f)
        with gzip.open(golden(f + ".gz"), "rb") as fi, open(dst, "wb") as fo:
            shutil.copyfileobj(fi, fo)
        out[f] = dst
    return out


@pytest.fixture(scope="session")
def port():
    from oracle import oracle as O
    if not os.path.exists(O.PORT_LIB):
        O.build_port()
    return O.PortOracle()


@pytest.fixture(scope="session")
def loprop(unpacked):
    from oracle import oracle as O
    return O.read_potfile(unpacked["loprop_solvated_20.pot"])


@pytest.fixture(scope="session")
def fmuls_golden():
    return np.loadtxt(golden("fmuls_loprop_solvated_20.txt.gz"))


@pytest.fixture(scope="session")
def fmm_errors_golden():
    import csv
    with gzip.open(golden("ref_fmm_errors.csv.gz"), "rt") as f:
        rows = list(csv.reader(f))
    hdr = rows[0][1:]
    data = np.array([[float(x) for x in r[1:]] for r in rows[1:]])
    return {h: data[:, i] for i, h in enumerate(hdr)}


def have_gpu():
    try:
        import cabi
        return cabi.device_count() > 0
    except Exception:
        return False


@pytest.fixture(scope="session")
def gpu():
    if not have_gpu():
        pytest.fail("test marked gpu but no CUDA device is usable (libcppe_gpu.so built?)")
    return True
