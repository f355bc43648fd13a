import os
import sys

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
sys.path.insert(0, HERE)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

from pkgload import pkg  # noqa: E402

GOLDEN = os.path.join(HERE, "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the GB300 kernels)")


@pytest.fixture(scope="session")
def P():
    return pkg()


@pytest.fixture(scope="session")
def built(P):
    """libcasoff.so and the CLI, compiled in-tree (nvcc cross-compiles without a GPU)."""
    return P.build()


@pytest.fixture(scope="session")
def oracle_bins():
    """(oracle port, reference binary or None)."""
    import build_oracle
    return build_oracle.build(with_reference=True)


@pytest.fixture(scope="session")
def oracle(oracle_bins):
    return oracle_bins[0]


@pytest.fixture(scope="session")
def reference(oracle_bins):
    return oracle_bins[1]


def golden_cases():
    return sorted(d for d in os.listdir(GOLDEN) if os.path.isdir(os.path.join(GOLDEN, d)))


def golden_input(case, tmpdir):
    """The case's input file with line 1 pointing at its genome; returns the path."""
    d = os.path.join(GOLDEN, case)
    lines = open(os.path.join(d, "input.txt")).read().split("\n")
    lines[0] = os.path.join(d, lines[0])
    path = os.path.join(str(tmpdir), f"{case}_input.txt")
    with open(path, "w") as f:
        f.write("\n".join(lines))
    return path
