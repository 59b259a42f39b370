"""CPU checks of the C ABI boundary: the shared library loads and exports every entry point that
include/bats_gb300.h declares, with the signatures the Python binding uses. No kernel is launched."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "bats_gb300.h")


def declared_symbols():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(bats_[a-z0-9_]+)\s*\(", src)))


@pytest.fixture(scope="module")
def lib():
    from bats_gb300 import _lib
    if not os.path.exists(_lib.LIB_PATH):
        from bats_gb300.build import build
        build()
    return ctypes.CDLL(_lib.LIB_PATH)


def test_header_declares_entry_points():
    syms = declared_symbols()
    assert "bats_lif_forward_fc" in syms and "bats_pre_errors" in syms
    assert len(syms) >= 20


def test_library_exports_every_declared_symbol(lib):
    missing = [s for s in declared_symbols() if not hasattr(lib, s)]
    assert not missing, missing


def test_python_binding_covers_every_declared_symbol():
    from bats_gb300 import _lib
    missing = [s for s in declared_symbols() if s not in _lib.SIGNATURES]
    assert not missing, missing


_SCALARS = {"int": ctypes.c_int, "long long": ctypes.c_longlong, "float": ctypes.c_float,
            "double": ctypes.c_double, "size_t": ctypes.c_size_t, "unsigned": ctypes.c_uint}


def _strip_comments(src):
    return re.sub(r"//[^\n]*", "", re.sub(r"/\*.*?\*/", "", src, flags=re.S))


def _ctype_of(decl, is_return=False):
    """ctypes class for one C declaration ("const float* times", "int batch", "cudaStream_t stream"), or
    "pointer" for any data pointer (the binding passes those as void* or as a typed pointer)."""
    decl = " ".join(decl.replace("const ", " ").split())
    if is_return:
        base = decl
    else:
        base = decl.rsplit(" ", 1)[0] if " " in decl and not decl.endswith("*") else decl
    if "*" in decl or base.startswith("cudaStream_t"):
        return ctypes.c_char_p if is_return and base.startswith("char") else "pointer"
    base = base.strip()
    assert base in _SCALARS, f"unmapped C type {base!r} in {decl!r}"
    return _SCALARS[base]


def header_declarations():
    """{name: (return ctype, [parameter ctypes])} of every function the header declares."""
    src = _strip_comments(open(HEADER).read())
    out = {}
    for m in re.finditer(r"([A-Za-z_][A-Za-z0-9_ ]*\**)\s*\b(bats_[a-z0-9_]+)\s*\(([^)]*)\)\s*;", src):
        ret, name, params = m.group(1).strip(), m.group(2), " ".join(m.group(3).split())
        args = [] if params in ("", "void") else [_ctype_of(p.strip()) for p in params.split(",")]
        out[name] = (_ctype_of(ret, is_return=True), args)
    return out


def _same(binding_type, header_type):
    if header_type == "pointer":
        return binding_type is ctypes.c_void_p or (isinstance(binding_type, type)
                                                   and issubclass(binding_type, ctypes._Pointer))
    return binding_type is header_type


def test_binding_signatures_match_the_header():
    """Every ctypes signature of the binding has the header's parameter count, order and types (a drift
    would pass wrong values without any error)."""
    from bats_gb300 import _lib
    decls = header_declarations()
    assert set(decls) == set(declared_symbols())
    wrong = []
    for name, (ret, args) in decls.items():
        b_ret, b_args = _lib.SIGNATURES[name]
        if not _same(b_ret, ret) or len(b_args) != len(args) or not all(map(_same, b_args, args)):
            wrong.append(name)
    assert not wrong, wrong


@pytest.mark.parametrize("struct", ["BatsFcLayer", "BatsFcTrainLayer"])
def test_layer_structs_match_the_header(struct):
    from bats_gb300 import _lib
    src = _strip_comments(open(HEADER).read())
    body = re.search(r"typedef struct " + struct + r" \{(.*?)\} " + struct + ";", src, re.S).group(1)
    fields = []
    for line in body.split(";"):
        line = " ".join(line.replace("const ", " ").split())
        if not line:
            continue
        first, *rest = [d.strip() for d in line.split(",")]
        head, name0 = first.replace("*", "* ").rsplit(" ", 1)
        for nm in [name0] + rest:
            ptr = "*" in head or nm.startswith("*")
            kind = "pointer" if ptr else (head.strip() if head.strip().startswith("Bats") else _SCALARS[head.strip()])
            fields.append((nm.lstrip("*"), kind))
    mirror = getattr(_lib, struct)._fields_
    assert [f[0] for f in mirror] == [f[0] for f in fields]
    for (_, bt), (_, ht) in zip(mirror, fields):
        if isinstance(ht, str) and ht.startswith("Bats"):
            assert bt is getattr(_lib, ht)  # a nested struct of the header, mirrored by the same name
        else:
            assert _same(bt, ht)


def test_status_strings_and_version(lib):
    lib.bats_status_string.restype = ctypes.c_char_p
    lib.bats_abi_version.restype = ctypes.c_int
    assert lib.bats_abi_version() == 1
    assert lib.bats_status_string(0) == b"ok"
    assert b"workspace" in lib.bats_status_string(4)


def test_shape_validation_without_a_gpu(lib):
    """Argument checks happen on the host before any launch and return a status."""
    from bats_gb300 import _lib
    L = _lib.load()
    st = L.bats_lif_forward_fc(None, None, 0, None, 1, 2, 4, 3, 1.0, 1.0, 1.0, 1.0, None, None, None, None, None,
                               None, None)
    assert st == 1  # BATS_ERR_BAD_SHAPE: ld < n_post
    st = L.bats_sort_events(None, 2, 3, 0, 1.0, 1.0, None, None, None, None, None, None, None, 0, None, 0, None)
    assert st == 1
    assert b"sort_events" in L.bats_last_error()
    # batch 0 is a no-op
    assert L.bats_adam_step(None, None, None, 0, 0.9, 0.999, 1e-8, 1e-3, 0.1, 0.001, None, None, None, 0, 0, 0,
                            None) == 0
    # the ordered sort needs its order and the counts; the order entry point its buffers (BATS_ERR_NULL)
    st = L.bats_sort_events_counted_ordered(None, None, 4, 3, 2, 1.0, 1.0, None, None, None, None, None, None,
                                            None, 32, None, None, 0, None)
    assert st == 2 and b"pre_counts" in L.bats_last_error()
    st = L.bats_sort_events_counted_ordered(None, ctypes.c_void_p(16), 4, 3, 2, 1.0, 1.0, None, None, None, None,
                                            None, None, None, 32, None, None, 0, None)
    assert st == 2 and b"sample_order" in L.bats_last_error()
    assert L.bats_sample_order(None, 4, None, None) == 2
    assert L.bats_sample_order(None, 0, None, None) == 0  # empty batch: nothing to order
    assert L.bats_sample_order(None, -1, None, None) == 1


def test_workspace_queries(lib):
    from bats_gb300 import _lib
    L = _lib.load()
    assert L.bats_sort_events_workspace_bytes(4, 10, 3) == 0  # fits in shared memory
    assert L.bats_sort_events_workspace_bytes(4, 512, 30) == 0  # 15360 slots: the whole layer in shared memory
    assert L.bats_sort_events_workspace_bytes(256, 512, 30) == 256 * 15360 * 12  # large batch: 7680 items
    # layers above 1024 slots sort with 512 threads, whose counters leave 6720 items at two CTAs per SM
    assert L.bats_sort_events_workspace_bytes(256, 256, 30) == 256 * 7680 * 12
    assert L.bats_sort_events_workspace_bytes(256, 200, 30) == 0
    assert L.bats_sort_events_workspace_bytes(256, 1024, 1) == 0  # 256 threads: room for 7680 items
    # two 4-byte key and two 2-byte slot buffers per slot when the slots fit 16 bits, 4-byte slots above
    assert L.bats_sort_events_workspace_bytes(4, 1000, 30) == 4 * 30000 * 12
    assert L.bats_sort_events_workspace_bytes(2, 4000, 20) == 2 * 80000 * 16
    # 16 partial gradients, 256-byte aligned, then one flag per (partial, pre bucket of 32, 32 post neurons)
    parts = (16 * 800 * 784 * 4 + 255) // 256 * 256
    assert L.bats_weights_gradient_workspace_bytes(256, 800, 784, 16) == parts + 16 * 25 * 25 * 4
    assert L.bats_weights_gradient_workspace_bytes(256, 800, 784, 1) == 0
    # cursor heads: a float2 per (sample, neuron), then from the next 16-byte boundary a float4 per pair
    assert L.bats_cursor_heads_bytes(3, 5) == 128 + 15 * 16
    assert L.bats_cursor_heads_bytes(256, 800) == 256 * 800 * 24
    # one float partial per (event, post tile of 128)
    assert L.bats_pre_errors_workspace_bytes(2, 100, 300) == 2 * 100 * 3 * 4


def test_bucket_width_matches_the_header():
    """The Python layer sorts events into the buckets the gradient kernels read (BATS_GRAD_BUCKET_WIDTH)."""
    from bats_gb300 import kernels as K
    m = re.search(r"#define BATS_GRAD_BUCKET_WIDTH (\d+)", open(HEADER).read())
    assert m and int(m.group(1)) == K.BUCKET_WIDTH
