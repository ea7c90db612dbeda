"""Recipe that compiles the reference's own C++ AMEn extension (``torchttcpp``).

TEST AND BASELINE INFRASTRUCTURE ONLY. Nothing in ``torchtt_gb300`` imports this module. The
compiled reference (``torchttcpp``: ``amen_solve``, ``round_this``, ``dmrg_mv``, ``tt_full``,
registered at ``cpp/cpp_ext.cpp:24-29``) is the strongest oracle for the AMEn path and the timed CPU
baseline of ``bench.py --impl reference``. It is built from the reference's sources unmodified, with
the flags of the reference's own ``setup.py:50-62`` (``-O3 -std=c++17``); the reference is a
libtorch ``CppExtension`` (one translation unit; no cmake, no generated code).

Two places hold the sources:

* the reference tree (``$TORCHTT_REFERENCE``, default ``/root/reference``), in the development
  container. ``build()`` compiles it into ``oracle/_ref/`` with ``torch.utils.cpp_extension``;
* the reference's install in ``baseline/_ref/`` (``pip install --target baseline/_ref`` of the
  reference, plus the extension's sources that ``stage()`` copies beside it, plus its pure-Python
  dependency ``opt_einsum``). ``build_installed()`` compiles the extension there with ``g++``
  directly (no ninja), as ``baseline/_ref/torchttcpp<EXT_SUFFIX>``, for the machine it runs on,
  so the reference's package ``torchtt`` imports it. ``baseline/_ref`` is not committed.

Usage::

    python oracle/build_ref.py              # oracle/_ref/torchttcpp.so (development container)
    python oracle/build_ref.py installed    # baseline/_ref/torchttcpp<EXT_SUFFIX> (any host)
"""
import os
import shutil
import subprocess
import sys
import sysconfig

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
REF_ROOT = os.environ.get("TORCHTT_REFERENCE", "/root/reference")
OUT_DIR = os.path.join(HERE, "_ref")
INSTALL = os.path.join(ROOT, "baseline", "_ref")


def reference_present():
    return os.path.isfile(os.path.join(REF_ROOT, "cpp", "cpp_ext.cpp"))


def installed_present():
    """The reference's install with the extension's sources staged beside it."""
    return (os.path.isdir(os.path.join(INSTALL, "torchtt"))
            and os.path.isfile(os.path.join(INSTALL, "cpp", "cpp_ext.cpp")))


def build(verbose=False):
    """Compile (or reuse) the reference extension from the tree; return the ``torchttcpp`` module."""
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


def stage():
    """Copies the extension's sources (``cpp/*.h``, ``cpp/cpp_ext.cpp``) and ``opt_einsum`` into the
    reference's install in ``baseline/_ref`` (which ``pip install --target`` fills with the Python
    package only), so that a host without the reference tree can build and import it."""
    if not (reference_present() and os.path.isdir(os.path.join(INSTALL, "torchtt"))):
        return False
    dst = os.path.join(INSTALL, "cpp")
    os.makedirs(dst, exist_ok=True)
    for f in os.listdir(os.path.join(REF_ROOT, "cpp")):
        if f.endswith(".h") or f == "cpp_ext.cpp":
            shutil.copy2(os.path.join(REF_ROOT, "cpp", f), os.path.join(dst, f))
    if not os.path.isdir(os.path.join(INSTALL, "opt_einsum")):
        try:
            import opt_einsum
            shutil.copytree(os.path.dirname(opt_einsum.__file__), os.path.join(INSTALL, "opt_einsum"),
                            ignore=shutil.ignore_patterns("__pycache__", "tests"))
        except ImportError:
            pass
    return True


def installed_module_path():
    return os.path.join(INSTALL, "torchttcpp" + sysconfig.get_config_var("EXT_SUFFIX"))


def build_installed(verbose=False):
    """Compiles ``baseline/_ref/cpp/cpp_ext.cpp`` against this host's torch with ``g++`` (no ninja)
    unless the module for this host is newer than its sources; returns its path."""
    import torch
    from torch.utils import cpp_extension as ce
    if not installed_present():
        raise RuntimeError("the reference's install with staged sources is not in %s" % INSTALL)
    src = os.path.join(INSTALL, "cpp", "cpp_ext.cpp")
    out = installed_module_path()
    newest = max(os.path.getmtime(os.path.join(INSTALL, "cpp", f)) for f in os.listdir(os.path.join(INSTALL, "cpp")))
    if os.path.exists(out) and os.path.getmtime(out) >= newest:
        return out
    abi = int(bool(getattr(torch._C, "_GLIBCXX_USE_CXX11_ABI", True)))
    inc = ce.include_paths() + [sysconfig.get_paths()["include"], os.path.join(INSTALL, "cpp")]
    libs = ce.library_paths()
    cmd = [os.environ.get("CXX", "g++"), "-O3", "-std=c++17", "-w", "-shared", "-fPIC",
           "-DTORCH_EXTENSION_NAME=torchttcpp", "-DTORCH_API_INCLUDE_EXTENSION_H",
           "-D_GLIBCXX_USE_CXX11_ABI=%d" % abi]
    cmd += ["-I" + p for p in inc] + [src, "-o", out + ".tmp"]
    cmd += ["-L" + p for p in libs] + ["-Wl,-rpath," + p for p in libs]
    cmd += ["-lc10", "-ltorch", "-ltorch_cpu", "-ltorch_python", "-Wl,--no-as-needed", "-lm"]
    if verbose:
        print(" ".join(cmd))
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("reference extension build failed:\n%s\n%s" % (r.stdout[-4000:], r.stderr[-4000:]))
    os.replace(out + ".tmp", out)
    return out


def load_installed():
    """Imports the reference's installed package ``torchtt`` (with its compiled ``torchttcpp``) from
    ``baseline/_ref``; returns ``(torchtt or None, torchttcpp)``. ``torchtt`` is None when its
    Python dependencies are missing on this host; the compiled extension is still returned."""
    build_installed()
    if INSTALL not in sys.path:
        sys.path.insert(0, INSTALL)
    import torchttcpp  # noqa: E402  (the reference's compiled extension)
    try:
        import torchtt  # noqa: E402  (the reference's package, from its install)
    except ImportError:
        torchtt = None
    return torchtt, torchttcpp


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
    if len(sys.argv) > 1 and sys.argv[1] == "installed":
        stage()
        print("built", build_installed(verbose=True))
    else:
        m = build(verbose=True)
        print("built", m.__file__)
