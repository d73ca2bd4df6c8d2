"""CPU oracles for the MC kinetics step (test infrastructure).

Everything under ``oracle/`` is the checker, never the product: only the test
suite, ``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py`` may
import it.  The library under ``mcluminescence_gb300`` runs on the GPU only and
never calls into this package.

Modules
-------
kinetics_k   FP64 restatement of the reference's event-driven KMC loop
             (src/class/simulate.py, tl_trap_lab.py, engine.py).
bernoulli    FP64 restatement of the fixed-dt Bernoulli kinetics (the batched
             mode), fed either injected uniforms or the Philox stream.
philox       Philox4x32-10 (Salmon et al., SC'11) in vectorised numpy.
mt19937      uniform stream of numpy's legacy RandomState (MT19937) used by
             the reference, for injected-uniform runs.
"""
