"""CPU checks of the C-ABI libraries: they build, load, and export every
symbol their headers declare -- include/hdc_gb300.h by libhdc_gb300.so,
include/hdc_synth.h by libhdc_synth.so (no compute call needs a GPU here)."""
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions(headers=("hdc_gb300.h",)):
    names = []
    for h in headers:
        src = open(os.path.join(ROOT, "include", h)).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        names += re.findall(r"^[A-Za-z_][\w \*]*?\b(hdc_\w+)\s*\(", src, flags=re.M)
    return sorted(set(names))


def test_header_declares_entry_points():
    names = declared_functions()
    assert "hdc_encode_segments" in names and "hdc_search_plain" in names and "hdc_bundle" in names


def test_library_exports_every_declared_symbol(hdc):
    lib = hdc.lib()
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_binding_covers_header(hdc):
    bound = {name for name, _, _ in hdc.SIGNATURES}
    assert set(declared_functions()) <= bound


def test_every_header_is_checked():
    assert sorted(h for h in os.listdir(os.path.join(ROOT, "include")) if h.endswith(".h")) == \
        ["hdc_gb300.h", "hdc_synth.h"]


def test_synth_library_exports_its_header():
    import build as pkg_build
    pkg_build.build_synth()
    import hdc_synth
    names = declared_functions(("hdc_synth.h",))
    assert names == ["hdc_synth_copies", "hdc_synth_reads", "hdc_synth_tree"]
    assert all(hasattr(hdc_synth.lib(), n) for n in names)
    assert {n for n, _, _ in hdc_synth.SIGNATURES} == set(names)


def test_product_library_holds_no_workload_generator(hdc):
    assert not any(hasattr(hdc.lib(), n) for n in declared_functions(("hdc_synth.h",)))


def test_status_strings(hdc):
    lib = hdc.lib()
    assert lib.hdc_status_string(0) == b"ok"
    assert lib.hdc_status_string(2) == b"value range"


def test_context_rejects_bad_sizes_without_gpu(hdc):
    import ctypes
    h = ctypes.c_void_p()
    assert hdc.lib().hdc_context_create(0, 8, 150, 10, ctypes.byref(h)) == 1
    assert b"dim" in hdc.lib().hdc_last_error()
    assert hdc.lib().hdc_context_create(1024, 17, 150, 10, ctypes.byref(h)) == 1
    assert hdc.lib().hdc_context_create(1024, 8, 0, 10, ctypes.byref(h)) == 1


def test_null_context_is_an_error(hdc):
    lib = hdc.lib()
    assert lib.hdc_norms(None, None, 2, 0, None, None, None) == 1
    assert lib.hdc_search_workspace_bytes(None, 1, 1, 1) == 0
    assert lib.hdc_num_windows(None, 500) == 0


def test_beam_search_split_argument_checks_without_gpu(hdc):
    """hdc_beam_search_split rejects a null context before any device work."""
    lib = hdc.lib()
    args = [None, None, None, 4, None, 0, None, None, 10, None, None, None, 1, 0, 6, 5, 0.0, 0, None, None, None,
            None]
    assert lib.hdc_beam_search_split(*args) == 1
    assert b"null context" in lib.hdc_last_error()
