"""Recipe that compiles the reference's own C++ AMEn extension into ``oracle/_ref/``.

TEST INFRASTRUCTURE ONLY. Nothing in ``torchtt_gb300`` imports this module. The compiled
reference (``torchttcpp``: ``amen_solve``, ``round_this``, ``dmrg_mv``, ``tt_full``, registered at
``cpp/cpp_ext.cpp:24-29``) is the strongest oracle available for the AMEn path: it is built from the
reference's sources where they lie, unmodified, with the flags of the reference's own ``setup.py:50-62``
(``-O3 -std=c++17``), through ``torch.utils.cpp_extension`` (the reference is a libtorch
``CppExtension``; no cmake, no generated code).

The reference tree is only present in the development container, so ``oracle/_ref`` exists only
there; the GPU host, which has no copy of the reference, falls back to the numpy restatement in
``oracle/amen.py``.

Usage::

    python oracle/build_ref.py            # builds oracle/_ref/torchttcpp*.so
"""
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REF_ROOT = os.environ.get("TORCHTT_REFERENCE", "/root/reference")
OUT_DIR = os.path.join(HERE, "_ref")


def reference_present():
    return os.path.isfile(os.path.join(REF_ROOT, "cpp", "cpp_ext.cpp"))


def build(verbose=False):
    """Compile (or reuse) the reference extension; return the imported ``torchttcpp`` module."""
    if not reference_present():
        raise RuntimeError("reference sources not present at %s" % REF_ROOT)
    from torch.utils.cpp_extension import load
    os.makedirs(OUT_DIR, exist_ok=True)
    return load(name="torchttcpp",
                sources=[os.path.join(REF_ROOT, "cpp", "cpp_ext.cpp")],
                extra_include_paths=[os.path.join(REF_ROOT, "cpp")],
                extra_cflags=["-O3", "-std=c++17", "-w"],
                build_directory=OUT_DIR,
                verbose=verbose)


def load_reference_package():
    """Import the reference's Python package ``torchtt`` with the compiled extension importable.

    Returns ``(torchtt, torchttcpp)``. Only usable where the reference tree exists.
    """
    mod = build()
    sys.modules.setdefault("torchttcpp", mod)
    if REF_ROOT not in sys.path:
        sys.path.insert(0, REF_ROOT)
    import torchtt  # noqa: E402  (the reference package)
    return torchtt, mod


if __name__ == "__main__":
    m = build(verbose=True)
    print("built", m.__file__)
