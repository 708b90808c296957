"""Every module of the package and the benchmark imports on a machine without
a GPU (syntax and import-time errors surface in the CPU suite)."""

import importlib

import pytest


@pytest.mark.parametrize("mod", ["jaxsplat_gb300", "jaxsplat_gb300._lib", "jaxsplat_gb300._ops",
                                 "jaxsplat_gb300.session", "jaxsplat_gb300.batch",
                                 "jaxsplat_gb300.fit", "jaxsplat_gb300.warmstart",
                                 "jaxsplat_gb300.scenes", "jaxsplat_gb300.build", "bench"])
def test_module_imports(mod):
    importlib.import_module(mod)
