"""Host logic of the resumable EM/OSEM driver (iterative.em_checkpointed):
which saved states a call accepts.  The GPU runs themselves are in
tests/test_gpu_em.py."""
from pyraft_gb300 import iterative as IT

PARAMS = {"niter": 4, "nsubsets": 5, "method": 2, "shape": [64, 64],
          "image_corners": [-1.0, 1.0, 1.0, -1.0],
          "sinogram": [64.0, 60.0, 0.0, 1.0, 3.14159, -1.0, 1234.5, 98765.25]}


def test_matching_state_is_accepted():
    state = dict(PARAMS, subiteration=7, done=False, x=None)
    assert IT._state_mismatch(state, PARAMS) is None


def test_each_parameter_is_checked():
    for key, other in [("niter", 5), ("nsubsets", 4), ("method", 3), ("shape", [64, 65]),
                       ("image_corners", [-1.0, 1.0, 1.0, -0.5]),
                       ("sinogram", PARAMS["sinogram"][:-1] + [98765.5])]:
        state = dict(PARAMS, subiteration=3)
        state[key] = other
        assert IT._state_mismatch(state, PARAMS) == key


def test_fingerprint_compares_to_relative_rounding():
    fp = list(PARAMS["sinogram"])
    fp[-1] *= 1 + 1e-15                     # a rounding-level difference in the FP64 sums
    assert IT._state_mismatch(dict(PARAMS, sinogram=fp), PARAMS) is None
