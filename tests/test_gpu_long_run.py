"""The 1,048,576-particle dam break over its whole 1,000-substep run
(dam_break_1m, dt = 1/600 s) against the reference itself: every 100
substeps the SHA-256 of the GPU's whole state (float32 positions and
velocities, id order) equals that of the reference's unmodified CPU solver,
whose digests tests/golden/make_golden.py --long-run froze in
tests/golden/dam_break_1m_long.json. Equal digests mean a bit-exact run, so
the long-run statistics (FP64 mean density, centre of mass) are the
reference's too; they are checked against the frozen values beside."""
from __future__ import annotations

import hashlib
import json
from pathlib import Path

import numpy as np
import pytest

from computer_graphics_lab_00_gb300 import workloads as W
from computer_graphics_lab_00_gb300.fluid import FluidSolverGpu

pytestmark = pytest.mark.gpu

GOLDEN = Path(__file__).resolve().parent / "golden" / "dam_break_1m_long.json"


def state_digest(pos: np.ndarray, vel: np.ndarray) -> tuple[str, str]:
    return (hashlib.sha256(np.ascontiguousarray(pos, np.float32).tobytes()).hexdigest(),
            hashlib.sha256(np.ascontiguousarray(vel, np.float32).tobytes()).hexdigest())


@pytest.mark.parametrize("neighbour_kernel", [4, 5, 6])
def test_1m_dam_break_1000_substeps_is_the_reference_run(native, neighbour_kernel):
    golden = json.loads(GOLDEN.read_text())
    case = W.dam_break_1m()
    assert golden["particles"] == case.count and golden["checkpoints"][-1]["substep"] == case.steps
    pos, vel = case.initial_state()
    with FluidSolverGpu(case.params, case.count) as solver:
        solver.set_tuning(neighbour_kernel=neighbour_kernel)
        solver.upload(pos, vel)
        done = 0
        for row in golden["checkpoints"]:
            solver.run(case.dt, row["substep"] - done)
            done = row["substep"]
            gp, gv = solver.state()
            assert state_digest(gp, gv) == (row["pos_sha256"], row["vel_sha256"]), f"substep {done}"
            st = solver.stats()
            np.testing.assert_allclose(st.mean_density, row["mean_density"], rtol=1e-12)
            np.testing.assert_allclose(list(st.centre_of_mass), row["centre_of_mass"], rtol=1e-12)
