"""CPU oracle for the lentil far-field MFT diffraction path.

TEST INFRASTRUCTURE ONLY.  Nothing in the shipped package imports this
module; only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline /
reference legs of ``bench.py`` use it, and there only as the checker or as
the timed CPU baseline.

``oracle.lentil_oracle`` restates, in plain numpy/scipy, the algorithms of
lentil 0.8.8 on the hot path (``lentil/fourier.py``, ``lentil/propagate.py``,
``lentil/field.py``, ``lentil/extent.py``, ``lentil/wavefront.py``,
``lentil/plane.py``, ``lentil/helper.py``, ``lentil/util.py``,
``lentil/detector.py``).  Every function cites the reference file:line it
follows.  Parity of the restatement is pinned by ``tests/test_oracle_golden.py``
against golden vectors that ``tests/golden/make_golden.py`` produced by running
lentil 0.8.8 itself on seeded inputs.
"""
