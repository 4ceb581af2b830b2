"""CPU oracle for the DNS-aided LES hot path — TEST INFRASTRUCTURE ONLY.

This package restates, in float64 NumPy, the algorithm of the reference
(agdestein/ExactClosure.jl, module ``NavierStokes`` in ``src/N.jl``) for the
periodic staggered-grid Navier–Stokes step, its FFT pressure projection, its
discrete filters and its exact-closure commutator.  Every function cites the
reference file:line it follows.

Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline legs of
``bench.py`` may import this package, and only as the reference the CUDA
results are compared with (or as the timed CPU baseline).  The product path (``libexc.so`` behind the C ABI) never
calls it and has no CPU fallback.

Parity pinning.  The reference is Julia and Julia is absent on every machine
this project runs on, and the reference ships no golden vectors.  The oracle
is pinned by (1) ``oracle.literal`` — a loop-for-loop restatement of the
reference's lazy-field code with its 1-based ``mod1`` indexing, run on small
grids — and (2) the reference's recorded known answers: the exact
"classic+flux+div" closure reproduces the filtered DNS to round-off
(``navierstokes.jl:33``, 5.69e-15) and ``randomfield`` is divergence free
(``navierstokes-test.jl:10-29``).  Parity with the reference's own outputs on
identical inputs is therefore pinned only through these invariants.
"""
