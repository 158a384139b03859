import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a) and the built extension")


@pytest.fixture(scope="session")
def golden():
    import numpy as np

    return np.load(os.path.join(ROOT, "tests", "golden", "reference_golden.npz"), allow_pickle=False)


@pytest.fixture(scope="session")
def dgolden():
    """Directional-regularisation and gradient-orthogonal fixtures."""
    import numpy as np

    return np.load(os.path.join(ROOT, "tests", "golden", "directional_golden.npz"), allow_pickle=False)


@pytest.fixture(scope="session")
def cgolden():
    """Fixtures at the benchmark configurations' sizes (make_golden.py --configs)."""
    import numpy as np

    return np.load(os.path.join(ROOT, "tests", "golden", "config_golden.npz"), allow_pickle=False)


@pytest.fixture(scope="session")
def agolden():
    """ADMM fixtures (make_golden.py --admm)."""
    import numpy as np

    return np.load(os.path.join(ROOT, "tests", "golden", "admm_golden.npz"), allow_pickle=False)


ADMM_CASES = ("admm_const", "admm_sched", "admm_adapt", "admm_loose")


def admm_kwargs(g, name):
    """The solver kwargs an ADMM fixture case was recorded with (besides the
    exact inner solver); x0 as the name of its start vector."""
    import ast

    out = {}
    for k, v in zip(g[f"{name}_kwargs_keys"], g[f"{name}_kwargs_vals"]):
        k, v = str(k), str(v)
        try:
            out[k] = ast.literal_eval(v)
        except (ValueError, SyntaxError):
            out[k] = v
    return out


class AffineBox:
    """A stand-in for the reference's BoundingBox built from its recorded
    affine maps: project / project_vectors / reproject / reproject_vectors."""

    def __init__(self, world_to_local, local_to_world, local_rotation):
        import numpy as np

        self.w2l = np.asarray(world_to_local, dtype=float)
        self.l2w = np.asarray(local_to_world, dtype=float)
        self.rot = np.asarray(local_rotation, dtype=float)

    @staticmethod
    def _affine(m, xyz):
        import numpy as np

        xyz = np.asarray(xyz, dtype=float)
        hom = np.ones((xyz.shape[0], 4))
        hom[:, :3] = xyz
        return (m @ hom.T).T[:, :3]

    def project(self, xyz):
        return self._affine(self.w2l, xyz)

    def reproject(self, xyz):
        return self._affine(self.l2w, xyz)

    def project_vectors(self, v):
        return (self.rot @ v.T).T

    def reproject_vectors(self, v):
        return (self.l2w[:3, :3] @ v.T).T
