"""The Python host binding (mkpp_gb300/api.py MechanismContext), on any host.

MechanismContext mirrors the reference's C++ wrapper (host_api/mkpp.hpp.j2):
a handle per context and an exception for every non-success status.  Creating
and binding make no CUDA call, so everything up to the first computing call
is checked here: metadata lookups, array validation, the C ABI's argument
errors surfacing as MkppError with the library's "FATAL ERROR" message, and,
without a GPU, MKPP_ERROR_DEVICE from the first call that computes.
"""
import numpy as np
import pytest

MECH = "chapman"


@pytest.fixture(scope="module")
def api():
    from mkpp_gb300 import api, build

    try:
        build.build((MECH,))
    except RuntimeError as e:  # no nvcc
        pytest.skip(str(e))
    return api


def _gpu():
    try:
        import torch

        return torch.cuda.is_available()
    except Exception:  # noqa: BLE001
        return False


def test_metadata_lookups(api):
    ctx = api.MechanismContext(MECH, 4)
    try:
        assert ctx.species_index("O3") == 2 and ctx.species_index("M") == 3
        assert ctx.photolysis_index("J_2") == 1
        with pytest.raises(api.MkppError) as e:
            ctx.species_index("XYZ")
        assert e.value.code == -106
        assert ctx.sizes.species == 4 and ctx.sizes.reactions == 4
    finally:
        ctx.close()


def test_array_validation_and_argument_errors(api):
    n = 4
    ctx = api.MechanismContext(MECH, n)
    try:
        conc = np.ones((4, n))
        t, p, rho = np.full(n, 300.0), np.full(n, 1e5), np.full(n, 2.4e19)
        with pytest.raises(TypeError):
            ctx.set_state(conc.astype(np.float32), t, p, rho)
        with pytest.raises(TypeError):
            ctx.set_state(np.asfortranarray(np.ones((4, n)))[:, ::2], t, p, rho)
        with pytest.raises(ValueError):
            ctx.set_state(np.ones((3, n)), t, p, rho)
        with pytest.raises(api.MkppError) as e:
            ctx.set_state(conc, np.array([300.0, -1.0, 300.0, 300.0]), p, rho)
        assert e.value.code == -103 and "FATAL ERROR" in str(e.value)
        ctx.set_state(conc, t, p, rho)
        with pytest.raises(api.MkppError) as e:
            ctx.set_rate_parameters(np.ones((3, n)))
        assert e.value.code == -103
        ctx.set_rate_parameters(np.zeros((2, n)))
        with pytest.raises(api.MkppError) as e:
            ctx.integrate(0.0)
        assert e.value.code == -103
        with pytest.raises(api.MkppError) as e:
            ctx.cell_stats()
        assert e.value.code == -104
    finally:
        ctx.close()


def test_first_computing_call(api):
    n = 4
    ctx = api.MechanismContext(MECH, n)
    try:
        conc = np.full((4, n), 1e9)
        ctx.set_state(conc, np.full(n, 300.0), np.full(n, 1e5), np.full(n, 2.4e19))
        ctx.set_rate_parameters(np.zeros((2, n)))
        if _gpu():
            ctx.integrate(60.0)
            assert (ctx.cell_stats()[0] == 0).all()
        else:
            with pytest.raises(api.MkppError) as e:
                ctx.integrate(60.0)
            assert e.value.code == -107 and "MKPP_ERROR_DEVICE" in str(e.value)
            assert (conc == 1e9).all()
    finally:
        ctx.close()
