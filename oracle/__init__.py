"""CPU FP64 oracle for the TemGymCore ray / beamlet-field hot path.

TEST INFRASTRUCTURE ONLY.  This package is the checker, never the product:
only ``tests/``, ``__graft_entry__.smoke()`` and the ``cpu_baseline`` /
``--impl reference`` legs of ``bench.py`` may import it.  The product
(``temgymcore_gb300``) must never import, call or fall back to anything here.

It is a NumPy restatement of the reference package ``temgym_core`` (pure
Python on JAX, which is not installable in this environment).  Every function
cites the reference ``file:line`` it follows.  The restatement is pinned
against the reference's own known-answer tests and README golden values
(``tests/golden/``, generated by ``tests/golden/make_golden.py``).

Model specification used by the oracle and by the tests: a list of dicts,
each with a ``"kind"`` key (``"lens"``, ``"scanner"``, ``"descanner"``,
``"deflector"``, ``"biprism"``, ``"rotator"``, ``"thicklens"``,
``"aperture"``, ``"plane"``, ``"detector"``, ``"scangrid"``, ``"source"``)
and that component's reference field names.
"""
from .rays import (  # noqa: F401
    ORay, run_to_end, run_iter, component_matrix, model_abcd, solve_model,
    propagate, apply_component,
)
from .grid import (  # noqa: F401
    pixels_to_metres_transform, metres_to_pixels_mat, metres_to_pixels,
    pixels_to_metres, into_image, grid_coords, round_to_int32,
)
from .phase import two_prod, reduce_2pi_dd, phase_offset_exact  # noqa: F401
