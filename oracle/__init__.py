"""CPU oracle for the MPS gate-application path (test infrastructure only).

Nothing in the product package imports this folder. Only ``tests/``,
``__graft_entry__.smoke()`` and the CPU-baseline legs of ``bench.py`` use it,
and only as the checker (or, for the baseline, as the CPU implementation that
is timed); the CUDA path never routes through it.

Contents:
  ref_mps   NumPy restatement of mpsim's MPS algorithm (mpsim/core.py,
            mpsim/gates.py) in complex64 and complex128.
  dense     dense state-vector simulator (stands in for Cirq, which the
            reference's own tests use as their oracle).
  tn_shim   restatement of the subset of TensorNetwork 0.2.1 that mpsim calls,
            used only to execute the reference's own ``core.py`` unmodified
            when the golden fixtures are generated.
"""
