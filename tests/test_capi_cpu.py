"""C-ABI checks that need no GPU: the library loads, exports every function
declared in include/*.h, and argument errors are reported without a device
(no compute calls here)."""
import ctypes as C
import os
import re

import afivo_gpu as ag

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = []
    inc = os.path.join(ROOT, "include")
    for f in sorted(os.listdir(inc)):
        if not f.endswith(".h"):
            continue
        src = open(os.path.join(inc, f)).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        names += re.findall(r"^\s*(?:const\s+)?[a-z_]+\s*\*?\s*(afg_[a-z0-9_]+)\s*\(", src, flags=re.M)
    return sorted(set(names))


def test_header_declares_entry_points():
    names = declared_functions()
    for must in ("afg_init", "afg_tree_sync", "afg_mg_vcycle", "afg_mg_fmg", "afg_mg_solve"):
        assert must in names


def test_library_exports_all_declared(gpu_lib):
    lib = C.CDLL(ag.LIB_PATH)
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_null_context_errors(gpu_lib):
    lib = ag.load_library()
    assert lib.afg_tree_sync(None, None, 1, 0) == ag.AFG_ERR_ARG
    assert lib.afg_finalize(None) == ag.AFG_ERR_ARG
    assert lib.afg_last_error(None) == b"null context"
    assert lib.afg_launch_count(None) == 0
