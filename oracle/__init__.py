"""CPU oracle for the USBS hot path: a NumPy/SciPy FP64 restatement of the reference.

This package is TEST INFRASTRUCTURE. Only ``tests/``, ``__graft_entry__.smoke()``
and the CPU-baseline leg of ``bench.py`` may import it, and only as the checker
(or as the timed CPU baseline).  The product package ``usbs_gb300`` never imports
it and never falls back to it.

Parity status: UNPINNED against the reference's own run.  The reference is JAX
(rangell/usbs, ``solver/*.py``, ``utils/*.py``); JAX is not installed where this
was written, and the reference ships no golden vectors or known-answer tests.
The oracle is therefore pinned by mathematics instead (analytic Laplacian
spectra, the MaxCut SDP value of complete graphs, the closed-form A(.)/A*(.)
adjoint identity, CGS orthogonality), see ``tests/test_oracle.py``.

Two inputs of the reference come from ``jax.random`` streams that cannot be
reproduced without JAX: the Lanczos start vector ``q0`` (``solver/usbs.py:691``,
``solver/cgal.py:108``) and the sketch test matrix ``Omega``
(``utils/maxcut_helpers.py:302``).  Both are explicit inputs here; the default
generator is :func:`oracle.rng.hash_normal`.  The Lanczos breakdown vector
(``solver/lanczos.py:110``, ``PRNGKey(i+1)``) uses ``hash_normal(i + 1, n)``.
"""
