"""The C-ABI library loads without a GPU and exports every function include/*.h declares."""
import ctypes as C
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = set()
    for h in os.listdir(os.path.join(ROOT, "include")):
        if not h.endswith(".h"):
            continue
        text = open(os.path.join(ROOT, "include", h)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"^\s*(?:const\s+)?[\w\s\*]+?\b(ne_\w+)\s*\(", text, flags=re.M):
            names.add(m.group(1))
    return names


def test_library_exports_every_declared_symbol(built):
    import narvalengine_gb300 as ne
    lib = C.CDLL(ne.LIB_PATH)
    names = declared_functions()
    assert "ne_render" in names and "ne_li_batch" in names and len(names) >= 15
    missing = [n for n in sorted(names) if not hasattr(lib, n)]
    assert not missing, missing
    # the ctypes table covers the same set
    from narvalengine_gb300 import _abi
    assert set(_abi.SIGNATURES) == names


def test_context_without_device_fails_cleanly(built):
    import narvalengine_gb300 as ne
    lib = ne.library()
    h = C.c_void_p()
    st = lib.ne_context_create(0, C.byref(h))
    if st == 0:  # a device is present: nothing to check here
        lib.ne_context_destroy(h)
        return
    assert st == -7 and not h.value  # NE_ERR_NO_DEVICE


def test_null_arguments_are_rejected(built):
    import narvalengine_gb300 as ne
    lib = ne.library()
    assert lib.ne_render(None, None, None, None) == -1
    assert lib.ne_trace_closest(None, None, 0, 0.0, 1.0, None) == -1
    assert lib.ne_scene_upload(None, None, None) == -1
    assert lib.ne_scene_host_load_json(None, None, None, None, 0) == -1
    assert lib.ne_context_set_cache_limit(None, 0) == -1


def test_every_entry_point_rejects_null_arguments(built):
    """Every function of the C ABI called with null pointers and zero sizes (no GPU needed):
    the status ones return an error, the others return without touching memory."""
    import narvalengine_gb300 as ne
    from narvalengine_gb300 import _abi
    lib = ne.library()
    for name, (ret, args) in sorted(_abi.SIGNATURES.items()):
        vals = []
        for a in args:
            if a in (C.c_void_p, C.c_char_p) or (isinstance(a, type) and issubclass(a, C._Pointer)):
                vals.append(None)
            elif a in (C.c_float, C.c_double):
                vals.append(0.0)
            else:
                vals.append(0)
        r = getattr(lib, name)(*vals)
        if ret is C.c_int32:
            assert r < 0, name
