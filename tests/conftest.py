import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "sde-sim-rs_gb300")
for p in (ROOT, PKG):
    if p not in sys.path:
        sys.path.insert(0, p)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as O
    O.build()
    return O


@pytest.fixture(scope="session")
def engine():
    import sde_sim_rs
    return sde_sim_rs


# Equation sets used across the tests.  The first three come from the
# reference's examples (examples/example.rs:11-14, examples/example.py:10-14,
# examples/example_gbm.py:13-15), written as the reference parses them.
GBM = ["dX = (0.05 * X) * dt + (0.2 * X) * dW1"]
EXAMPLE_RS = ["dX1 = ( sin(t) ) * dt + (0.01 * X1) * dW1 + (0.001 * X1) * dN1(0.5 * cos(t))",
              "X2 = max(X1 - 100.0, 0.0)"]
EXAMPLE_PY = ["dX0 = ( 2.0 * (0.5 - X0) ) * dt + ( 0.1 ) * dN1(X0)",
              "dX1 = ( 0.05 * X1 ) * dt + ( 0.2 * X1 ) * dW1 + ( 0.5 ) * dN1(X0)",
              "X2 = max(X1 - 100.0, 0.0)"]
EXAMPLE_GBM = ["dX1 = ( 0.05 * X1 ) * dt + ( 0.1 * X1) * dW1"]
HESTON = ["dv = (2 * (0.04 - max(v, 0))) * dt + (0.3 * max(v, 0)^0.5) * dW1",
          "dS = (0.03 * S) * dt + (-0.7 * max(v, 0)^0.5 * S) * dW1 + "
          "(0.714142842854285 * max(v, 0)^0.5 * S) * dW2"]
OU = ["dX = (2.0 * (0.5 - X)) * dt + (0.3) * dW1"]
