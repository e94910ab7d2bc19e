"""CPU restatement of the JaQMC VMC inner loop — TEST INFRASTRUCTURE ONLY.

This package is the parity oracle and the timed CPU baseline for the GB300
library in ``jaqmc_gb300``.  It is imported only by ``tests/``,
``__graft_entry__.smoke()`` and the ``cpu_baseline`` / ``--impl reference``
legs of ``bench.py``; the product path never routes through it.

What it restates (torch on CPU, float64 or float32):

* ``lap``        — value/Jacobian/Laplacian tangent algebra following the
                   forward-Laplacian rules of ``src/jaqmc/laplacian/primitives``.
* ``ferminet``   — FermiNet log|psi| (``src/jaqmc/app/molecule/wavefunction/ferminet.py``).
* ``psiformer``  — Psiformer log|psi| + simple e-e Jastrow
                   (``src/jaqmc/app/molecule/wavefunction/psiformer.py``).
* ``hamiltonian``— Coulomb potential and kinetic energy
                   (``src/jaqmc/app/molecule/hamiltonian.py``,
                   ``src/jaqmc/estimator/kinetic/_common.py``).
* ``mcmc``       — the all-electron Gaussian Metropolis-Hastings update with
                   externally supplied draws (``src/jaqmc/sampler/mcmc.py``).
* ``stats``      — mean/variance reduction, MAD/IQR clipping, the VMC
                   gradient algebra (``src/jaqmc/estimator/base.py``,
                   ``src/jaqmc/utils/clip.py``, ``src/jaqmc/estimator/loss_grad.py``).
* ``philox``     — Philox4x32-10 counter-based generator (integer-exact).

Parity status: the reference (JAX/Flax) cannot be imported where this code
runs, and it ships no golden numeric vectors for FermiNet/Psiformer log|psi|
or E_L.  The oracle is pinned by the reference's own known-answer and
property tests restated in ``tests/test_oracle_*.py`` (forward Laplacian ==
brute-force Hessian trace, analytic harmonic kinetic energy, slogdet rule,
antisymmetry, exact hydrogen-like energies).  Against reference-produced
vectors it is "parity unpinned".
"""
