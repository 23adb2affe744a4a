"""CPU FP64 oracle for the co-kriging hot path -- TEST INFRASTRUCTURE ONLY.

This package is the checker, never the product: only ``tests/``,
``__graft_entry__.smoke()`` and the ``cpu_baseline`` / ``--impl reference``
legs of ``bench.py`` may import it.  The product path (``gempy_gb300``) never
imports it and has no CPU fallback.

What it restates.  The arithmetic of GemPy's implicit potential-field
co-kriging lives in the external package ``gempy_engine`` (pinned
``gempy_engine>=2026.0.3`` in ``requirements/requirements.txt:2``), which is not
vendored in the reference and cannot be installed here.  The oracle therefore
restates the published method -- de la Varga, Schaaf & Wellmann 2019, "GemPy
1.0", GMD 12:1-32 (``CITATION.cff:1-16``), built on Lajaunie et al. 1997 and
Calcagno et al. 2008 (``docs/source/index.rst:76-82``) -- in plain numpy/scipy
FP64, and anchors parity on the reference's own call site
(``gempy/API/compute_API.py:68-73``), its input layout
(``gempy/modules/data_manipulation/_engine_factory.py:14-58``) and its
known-answer tests:

* pinned, ids: the anticline cube-corner lithology ids ``[3,3,3,3,1,1,1,1]``
  (``test/test_modules/test_grids/test_custom_grid.py:44-65``), reproduced
  from the bundled ``examples/data/input_data/jan_models/model2_*.csv`` inputs
  with the input transform pinned by the reference's approved model JSON
  (``test_custom_grid.test_custom_grid.verify/fold.approved.txt:108-126``);
* pinned, field: the 51-value scalar-field approval file of the anticline's
  finest octree level (``test/test_model_types/test_example_models_I.py:41-53``)
  under the reference's comparator ``np.allclose(rtol=1e-5, atol=1e-5)``
  (``test/verify_helper.py:70-103``), octree point order included.  The
  block-level conventions (``kriging`` module docstring) were chosen with this
  file; the fault-model approval file (``test_example_models_I.py:56-68``)
  judges them independently;
* pinned, field and refinement: the combination model's approval file
  (``test_example_models_I.py:71-88``), which also fixed the form of the
  octree's interpolation-error refinement (``octree`` module docstring);
* pinned, counts: the combination model's marching-cubes vertex counts
  (``test/test_modules/test_marching_cubes.py:44-47``, ``mesh`` module);
* pinned, value: the two-layer model's gravity, -1624.1714
  (``test/test_modules/test_geophysics/test_gravity.py:89``, ``gravity``).

Modules: ``covariance`` (kernel functions), ``kriging`` (matrix build, solve,
evaluation), ``segmentation`` (sigmoid ids, series masks), ``octree`` (corner
and interpolation-error refinement), ``pipeline`` (multi-series compute_model
restatement), ``mesh`` (marching cubes), ``gravity`` (prism forward gravity on
centred grids, pinned by the reference's two-layer gravity value), ``mlp``
(the preconditioner network).
"""
from . import covariance, kriging, segmentation, octree, pipeline  # noqa: F401
