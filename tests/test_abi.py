"""The C-ABI library builds, loads without a GPU and exports every declared symbol."""
import ctypes
import glob
import os
import re

from tests.conftest import ROOT


def declared_functions():
    names = []
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        src = open(h).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        names += re.findall(r"^\s*(?:const\s+)?[A-Za-z_][A-Za-z0-9_]*\s*\**\s+\**(pf_[A-Za-z0-9_]+)\s*\(",
                            src, flags=re.M)
    return sorted(set(names))


def test_header_declares_entry_points():
    names = declared_functions()
    assert "pf_transport_tdb" in names and "pf_transport_tdb_dev" in names


def test_library_exports_all_declared_symbols(built_lib):
    lib = ctypes.CDLL(built_lib)
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_python_binding_covers_header(built_lib):
    from phinfortran_gb300 import _abi
    _abi.load()
    assert set(declared_functions()) <= set(_abi.SIGNATURES)


def test_version_and_error_without_gpu(built_lib):
    from phinfortran_gb300 import _abi
    lib = _abi.load()
    assert lib.pf_version() == 1
    # argument validation runs on the host: no device needed
    rc = lib.pf_transport_tdb(0, 1, 1, 1, 1, *([None] * 8), 0, None, None, None,
                              0.0, 0.0, 1.0, 1e-14, 10, 0, None, None, None, None)
    assert rc == -1
    assert b"positive" in lib.pf_last_error()


def test_argument_validation_of_later_entries_without_gpu(built_lib):
    """The full-Hamiltonian, tight-binding and Buttiker-probe entries reject
    bad sizes on the host before touching a device."""
    from phinfortran_gb300 import _abi
    lib = _abi.load()
    rc = lib.pf_gen_dyn(0, 1, 1, 1, 1, 3, 3, None, None, 0, None, None, None, None, 1, None, 1, None)
    assert rc == -1 and b"positive" in lib.pf_fullh_last_error()
    rc = lib.pf_gen_dyn(4, 1, 1, 3, 2, 9, 9, None, None, 0, None, None, None, None, 1, None, 1, None)
    assert rc == -1 and b"multiple of nz" in lib.pf_fullh_last_error()
    rc = lib.pf_buttiker_tdb(4, 4, 4, 1, 1, *([None] * 8), 1, None, None, None, *([None] * 6),
                             0.0, 0.0, 10.0, 1e-14, 10, *([None] * 7), None)
    assert rc == -1 and b"two device layers" in lib.pf_buttiker_last_error()
    rc = lib.pf_buttiker_tdb(64, 4, 4, 3, 1, *([None] * 8), 1, None, None, None, *([None] * 6),
                             0.0, 0.0, 10.0, 1e-14, 10, *([None] * 7), None)
    assert rc == -3


def test_argument_validation_of_mode_entries_without_gpu(built_lib):
    """The per-mode entry wants its three per-mode outputs together, and both
    mode entries reject bad sizes on the host."""
    import ctypes as C

    from phinfortran_gb300 import _abi
    lib = _abi.load()
    kz = C.c_void_p(8)   # never dereferenced: the call is refused before any device work
    args = (4, 4, 4, 2, 1, *([None] * 8), 1, None, None, None, 0.0, 1e-6, 10.0, 1e-14, 10, 5e-3, 1.0, 1.0, 1,
            4, 4, None, 4, 4, None, None, None, None, None, None)
    rc = lib.pf_transport_tdb_modes_permode_dev(*args, kz, None, None, None, 0, None)
    assert rc == -1 and b"all given or all null" in lib.pf_modes_last_error()
    bad = (0,) + args[1:]
    rc = lib.pf_transport_tdb_modes_permode_dev(*bad, None, None, None, None, 0, None)
    assert rc == -1 and b"positive" in lib.pf_modes_last_error()
    rc = lib.pf_transport_tdb_modes_dev(*bad, None, 0, None)
    assert rc == -1 and b"positive" in lib.pf_modes_last_error()


def test_argument_validation_of_tensor_core_and_mixed_entries_without_gpu(built_lib):
    """The tensor-core GEMM refuses k above its exact-accumulation range, the
    mixed entry unknown lead arithmetics, the blocks entry bad sizes and the
    stage timer a query before any timed call -- all on the host."""
    from phinfortran_gb300 import _abi
    lib = _abi.load()
    rc = lib.pf_tc_zgemm_dev(ord("N"), ord("N"), 4, 4, 4096, 1.0, None, 4, 0, None, 4096, 0, 0.0, None, 4, 0, 1,
                             None, 0, None)
    assert rc == -3 and b"2048" in lib.pf_tc_last_error()
    rc = lib.pf_tc_zgemm_dev(ord("T"), ord("N"), 4, 4, 4, 1.0, None, 4, 0, None, 4, 0, 0.0, None, 4, 0, 1,
                             None, 0, None)
    assert rc == -1
    rc = lib.pf_transport_tdb_mixed_ex_dev(4, 4, 4, 2, 1, *([None] * 8), 1, None, None, None, 0.0, 1e-6, 10.0,
                                           1e-14, 10, 2, 7, None, None, None, None, 0, None)
    assert rc == -1 and b"lead_arith" in lib.pf_last_error()
    rc = lib.pf_transport_tdb_blocks_dev(0, 4, 4, 2, 1, *([None] * 8), 1, None, None, None, 0.0, 1e-6, 10.0,
                                         1e-14, 10, None, None, None, *([None] * 10), None, 0, None)
    assert rc == -1 and b"positive" in lib.pf_modes_last_error()
    import ctypes as C
    buf = (C.c_float * 3)()
    lib.pf_mixed_stage_timing(0)
    assert lib.pf_mixed_stage_times(buf, 3) == -1


def test_tiled_tuning_knobs_without_gpu(built_lib):
    """The large-block tuning knobs are validated and reported on the host:
    a panel width outside {0, 4, 8, 16, 32} is refused, a requested panel
    is narrowed when it does not fit in shared memory, and the batch is
    capped by the request and by the number of points."""
    import ctypes as C

    from phinfortran_gb300 import _abi
    lib = _abi.load()
    assert lib.pf_tiled_set_tuning(5, 0) == -1
    p, b = C.c_int(), C.c_int()
    try:
        assert lib.pf_tiled_set_tuning(32, 64) == 0
        assert lib.pf_tiled_layout(96, 96, 96, 1000, 0, C.byref(p), C.byref(b)) == 0
        assert (p.value, b.value) == (32, 64)
        assert lib.pf_tiled_layout(768, 768, 768, 10, 0, C.byref(p), C.byref(b)) == 0
        assert p.value <= 8 and b.value == 10
        assert lib.pf_tiled_set_tuning(0, 0) == 0
        assert lib.pf_tiled_layout(96, 96, 96, 1000, 0, C.byref(p), C.byref(b)) == 0
        assert p.value == 32 and b.value == 256
    finally:
        lib.pf_tiled_set_tuning(0, 0)


def test_tiled_circular_validation_without_gpu(built_lib):
    """The block-circulant entry checks its Bloch cells on the host: nl must
    equal nr and be a multiple of n_bloch_y * n_bloch_x, gr must be given;
    its workspace is the plain engine's plus the small-block engine's."""
    import ctypes as C

    from phinfortran_gb300 import _abi
    lib = _abi.load()
    ws = lib.pf_transport_tdb_tiled_circ_workspace_size
    plain = lib.pf_transport_tdb_tiled_workspace_size(96, 96, 96, 10, 1, 64, 0)
    assert ws(96, 96, 96, 10, 1, 64, 0, 2, 2) > plain
    assert ws(96, 96, 96, 10, 1, 64, 0, 5, 2) == 0
    assert ws(96, 96, 48, 10, 1, 64, 0, 2, 2) == 0
    assert ws(96, 96, 96, 10, 1, 64, 0, 0, 2) == 0
    assert ws(66, 66, 66, 10, 1, 64, 0, 33, 1) == 0     # phase table of the back transform
    gr = (C.c_double * 4)(*([6.283185307179586] * 4))
    args = [96, 96, 96, 10, 1] + [None] * 8 + [1, None, None, None, 0.0, 1e-5, 10.0, 1e-14, 100, 0]
    rc = lib.pf_transport_tdb_tiled_circ_dev(*args, 5, 2, gr, None, None, None, None, 0, None)
    assert rc == -1 and b"multiple" in lib.pf_tiled_last_error()
    rc = lib.pf_transport_tdb_tiled_circ_dev(*args, 2, 2, None, None, None, None, None, 0, None)
    assert rc == -1 and b"gr" in lib.pf_tiled_last_error()
    rc = lib.pf_transport_tdb_tiled_circ_dev(*args, 2, 2, gr, None, None, None, None, 0, None)
    assert rc == -1 and b"null block pointer" in lib.pf_tiled_last_error()
