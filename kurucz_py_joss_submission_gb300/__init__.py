"""GB300-native line-opacity and transfer path of synthe_py (PySynthe).

The package mirrors the reference's call surface for this path --
``cli.main``, ``engine.run_synthesis``, ``physics.line_opacity.compute_transp``
/ ``compute_asynth_from_transp`` and ``engine.radiative.solve_lte_spectrum`` --
on top of the C ABI of ``libkurucz_gb300.so`` (hand-written sm_103a kernels).
"""

__version__ = "1.0.0"

__all__ = ["__version__"]
