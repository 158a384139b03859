"""Host logic of the regularisation configuration (the reference's
_regularisation.py forms and errors).  CPU only."""
import numpy as np
import pytest

from loopstructural_gb300 import regularisation as R


def test_scalar_and_dict_forms():
    assert R.coerce_regularisation_config(0.3).isotropic == 0.3
    cfg = R.coerce_regularisation_config({"isotropic": 0.2, "directional": [{"weight": 1.0, "vector": np.ones((2, 3))}]})
    assert cfg.isotropic == 0.2 and len(cfg.directional) == 1
    assert cfg.directional[0].name == "directional regularisation 1"
    # a single directional mapping
    cfg = R.coerce_regularisation_config({"weight": 0.5, "direction": np.ones((2, 3))})
    assert cfg.isotropic is None and cfg.directional[0].weight == 0.5
    # the separate argument is appended
    t = R.DirectionalRegularisation(0.1, np.ones((2, 3)), "x")
    cfg = R.coerce_regularisation_config(0.1, [t, t])
    assert cfg.isotropic == 0.1 and len(cfg.directional) == 2


def test_errors():
    with pytest.raises(TypeError):
        R.coerce_regularisation_config(object())
    with pytest.raises(ValueError):  # a string is a numpy scalar: float() fails, as in the reference
        R.coerce_regularisation_config("abc")
    with pytest.raises(TypeError):
        R.coerce_directional_regularisation([0.1, 0.2])
    with pytest.raises(ValueError):
        R.coerce_directional_regularisation({"weight": 1.0})
    with pytest.raises(ValueError):
        R.coerce_directional_regularisation({"direction": np.ones((2, 3))})
    assert R.coerce_directional_regularisation(None) == ()
    assert R.coerce_directional_regularisation([]) == ()


def test_duck_typed_reference_objects():
    class Term:  # the reference's DirectionalRegularisation has these attributes
        def __init__(self):
            self.weight, self.direction, self.name = 0.4, np.zeros((1, 3)), "t"

    class Cfg:
        isotropic = 0.7
        directional = (Term(),)

    cfg = R.coerce_regularisation_config(Cfg())
    assert cfg.isotropic == 0.7 and cfg.directional[0].name == "t"
    assert R.coerce_directional_regularisation(Term())[0].weight == 0.4
