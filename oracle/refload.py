"""Load the reference quafu package with the reference qfvm module built by
oracle/build_ref.sh (test infrastructure only: golden-fixture generation in the
build container; the reference tree is not present on GPU machines).

Call ``load(qfvm_module=None)``: puts oracle/pystubs and the reference root on
sys.path, registers ``quafu.simulators.qfvm`` (the reference build by default,
or any module object passed in, e.g. the GB300 drop-in), then imports quafu.
"""
import glob
import importlib.util
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))


def _reference_root() -> str:
    """$QFVM_REFERENCE_ROOT, else the tree oracle/build_ref.sh last built from."""
    root = os.environ.get("QFVM_REFERENCE_ROOT")
    if root:
        return root
    try:
        with open(os.path.join(HERE, "_ref", "reference_root")) as f:
            return f.read().strip()
    except OSError:
        return ""


REFERENCE_ROOT = _reference_root()


def ref_qfvm_path():
    hits = glob.glob(os.path.join(HERE, "_ref", "qfvm*.so"))
    return hits[0] if hits else None


def available() -> bool:
    return bool(REFERENCE_ROOT) and os.path.isdir(os.path.join(REFERENCE_ROOT, "quafu")) and \
        ref_qfvm_path() is not None


def load_ref_qfvm():
    path = ref_qfvm_path()
    if path is None:
        raise RuntimeError("reference qfvm not built: run oracle/build_ref.sh")
    spec = importlib.util.spec_from_file_location("qfvm", path)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def load(qfvm_module=None):
    sys.dont_write_bytecode = True  # never write __pycache__ into the reference tree
    stubs = os.path.join(HERE, "pystubs")
    if stubs not in sys.path:
        sys.path.insert(0, stubs)
    if REFERENCE_ROOT not in sys.path:
        sys.path.insert(0, REFERENCE_ROOT)
    if qfvm_module is None:
        qfvm_module = load_ref_qfvm()
    sys.modules["quafu.simulators.qfvm"] = qfvm_module
    import quafu  # noqa: F401

    return quafu
