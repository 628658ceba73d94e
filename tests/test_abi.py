"""The C ABI library: builds for sm_103a, loads, and exports every entry point
that include/diffmpm_gb300.h declares (no GPU needed)."""
import ctypes
import re
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
HEADER = ROOT / "include" / "diffmpm_gb300.h"


def declared_functions():
    text = HEADER.read_text()
    return sorted(set(re.findall(r"^\s*(?:int|const char\*)\s+(mpm_\w+)\s*\(", text, re.M)))


def test_header_declares_entry_points():
    names = declared_functions()
    assert "mpm_create" in names and "mpm_step" in names and len(names) >= 15


def test_library_exports_every_declared_symbol(built):
    from diffmpm_gb300 import _lib
    lib = _lib.load()
    for name in declared_functions():
        assert hasattr(lib, name), name
    bound = {name for name, _, _ in _lib.SIGNATURES}
    assert set(declared_functions()) == bound


def test_abi_version(built):
    from diffmpm_gb300 import _lib
    assert _lib.load().mpm_abi_version() == 1


def test_create_rejects_bad_scheme_without_gpu(built):
    # argument validation happens before any device call
    from diffmpm_gb300 import _lib
    lib = _lib.load()
    d = _lib.MpmDesc()
    d.ndim = 2
    d.nelements[0] = d.nelements[1] = 2
    d.el_len[0] = d.el_len[1] = 0.5
    d.scheme = 7
    h = ctypes.c_void_p()
    rc = lib.mpm_create(ctypes.byref(d), ctypes.byref(h))
    assert rc == 1
    assert b"scheme" in lib.mpm_last_error(None)


def test_create_validates_dimension(built):
    """ndim 1 (Linear1D) and 2 only; a 1-D mesh takes direction 0 only."""
    from diffmpm_gb300 import _lib
    lib = _lib.load()
    d = _lib.MpmDesc()
    d.ndim = 3
    h = ctypes.c_void_p()
    assert lib.mpm_create(ctypes.byref(d), ctypes.byref(h)) == 5
    d.ndim = 1
    d.nelements[0] = 4
    d.el_len[0] = 0.25
    d.scheme = _lib.USF
    node = (ctypes.c_int32 * 1)(0)
    direction = (ctypes.c_int32 * 1)(1)
    vel = (ctypes.c_double * 1)(0.0)
    d.n_constraints = 1
    d.constraint_node, d.constraint_dir, d.constraint_velocity = node, direction, vel
    mats = (_lib.MpmMaterial * 1)()
    mats[0].type, mats[0].density, mats[0].E = 1, 1.0, 100.0
    d.n_materials, d.materials = 1, mats
    assert lib.mpm_create(ctypes.byref(d), ctypes.byref(h)) == 1
    assert b"dir must be 0 in 1-D" in lib.mpm_last_error(None)


def test_library_is_sm103a(built):
    from diffmpm_gb300 import _lib
    data = _lib.LIB_PATH.read_bytes()
    assert b"sm_103a" in data


def test_python_api_mirrors_reference_names():
    import diffmpm_gb300 as D
    for name in ("Mesh2D", "Particles", "Quadrilateral4Node", "MPMExplicit", "LinearElastic",
                 "SimpleMaterial", "Newtonian", "Constraint", "NodalForce", "ParticleTraction",
                 "Unit", "Linear", "Linear1D", "Mesh1D"):
        assert hasattr(D, name)


def test_invalid_scheme_raises_value_error():
    import numpy as np
    import diffmpm_gb300 as D
    mat = D.LinearElastic({"density": 1, "youngs_modulus": 1, "poisson_ratio": 0})
    el = D.Quadrilateral4Node((1, 1), 1, (1.0, 1.0), [])
    ps = D.Particles(np.full((1, 1, 2), 0.5), mat, np.zeros(1))
    mesh = D.Mesh2D({"particles": [ps], "elements": el})
    with pytest.raises(ValueError):
        D.MPMExplicit(mesh, 0.1, scheme="abc")


def test_missing_material_property_raises_key_error():
    import diffmpm_gb300 as D
    with pytest.raises(KeyError):
        D.LinearElastic({"density": 1, "youngs_modulus": 1})


def test_create_rejects_meshes_beyond_the_node_index_range(built):
    from diffmpm_gb300 import _lib
    lib = _lib.load()
    d = _lib.MpmDesc()
    d.ndim = 2
    d.nelements[0] = d.nelements[1] = 40000     # 1.6e9 nodes > 2^30
    d.el_len[0] = d.el_len[1] = 1.0
    h = ctypes.c_void_p()
    assert lib.mpm_create(ctypes.byref(d), ctypes.byref(h)) == 1
    assert b"too large" in lib.mpm_last_error(None)


def test_read_destinations_are_checked_before_the_library_writes():
    """A read into a caller's ``out`` must be refused when the library would
    write past it or scramble it: too few elements, a wrong dtype, a
    non-contiguous or read-only array (checked on the host, no GPU)."""
    import numpy as np
    from diffmpm_gb300.engine import _out_arg
    good = np.empty((10, 2), np.float32)
    p, dev = _out_arg(good, np.float32, 20)
    assert dev == 0 and p.value == good.ctypes.data
    with pytest.raises(ValueError, match="20 elements"):
        _out_arg(np.empty(10, np.float32), np.float32, 20)          # undersized
    with pytest.raises(ValueError, match="float32"):
        _out_arg(np.empty((10, 2), np.float64), np.float32, 20)     # float64
    with pytest.raises(ValueError):
        _out_arg(np.empty((10, 4), np.float32)[:, :2], np.float32, 20)   # strided view
    ro = np.empty(20, np.float32)
    ro.flags.writeable = False
    with pytest.raises(ValueError):
        _out_arg(ro, np.float32, 20)
    with pytest.raises(ValueError, match="int32"):
        _out_arg(np.empty(20, np.float32), np.int32, 20)            # integer field
    with pytest.raises(ValueError):
        _out_arg([0.0] * 20, np.float32, 20)                        # not an array


def test_output_enqueue_takes_the_destination_size():
    """mpm_output_enqueue is told how large the pinned destination is."""
    text = HEADER.read_text()
    decl = re.search(r"int mpm_output_enqueue\(([^)]*)\)", text, re.S).group(1)
    assert "size_t host_dst_bytes" in decl


def test_every_entry_point_refuses_a_null_handle(built):
    """Each call on a handle or batch checks the handle before it touches it or
    the device: a NULL handle gives MPM_ERR_INVALID (destroying NULL is a
    no-op, and the last-error calls of NULL give the creation error)."""
    from diffmpm_gb300 import _lib
    lib = _lib.load()
    no_op = {"mpm_destroy", "mpm_batch_destroy"}
    checked = 0
    for name, restype, argtypes in _lib.SIGNATURES:
        if restype is not ctypes.c_int or not argtypes or argtypes[0] is not ctypes.c_void_p:
            continue
        if name in ("mpm_host_free",):     # a host pointer, not a handle
            continue
        args = [None if t is ctypes.c_void_p or hasattr(t, "contents") or t is ctypes.c_char_p
                else t(0) for t in argtypes]
        rc = getattr(lib, name)(*args)
        assert rc == (0 if name in no_op else 1), (name, rc)
        checked += 1
    assert checked >= 30
    assert isinstance(lib.mpm_last_error(None), bytes)
    assert isinstance(lib.mpm_batch_last_error(None), bytes)


def test_c_program_links_and_sees_the_python_struct_layouts(built, tmp_path):
    """A plain C99 program (the shape of a cgo / FFI binding) compiles against
    the header, links against the library and calls it without a GPU; the
    layouts it reports for the descriptor, material and tuning structs are
    the ones the Python binding declares."""
    import shutil
    import subprocess
    from diffmpm_gb300 import _lib
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    structs = {"MpmDesc": _lib.MpmDesc, "MpmMaterial": _lib.MpmMaterial, "MpmTuning": _lib.MpmTuning}
    lines = ['#include <stddef.h>', '#include <stdio.h>', '#include <string.h>',
             '#include "diffmpm_gb300.h"', 'int main(void) {',
             '    if (mpm_abi_version() != MPM_ABI_VERSION) return 2;',
             '    if (mpm_step(NULL, 1, NULL) != MPM_ERR_INVALID) return 3;',
             '    MpmDesc d; memset(&d, 0, sizeof d);',
             '    d.ndim = 2; d.nelements[0] = d.nelements[1] = 2;',
             '    d.el_len[0] = d.el_len[1] = 0.5; d.scheme = 7;',
             '    MpmHandle* h = NULL;',
             '    if (mpm_create(&d, &h) != MPM_ERR_INVALID || h != NULL) return 4;',
             '    if (!strstr(mpm_last_error(NULL), "scheme")) return 5;']
    for s in structs:
        lines.append(f'    printf("{s} size %zu\\n", sizeof({s}));')
        for f, _ in structs[s]._fields_:
            lines.append(f'    printf("{s} {f} %zu\\n", offsetof({s}, {f}));')
    lines += ['    return 0;', '}']
    src = tmp_path / "binding.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "binding"
    lib_dir = _lib.LIB_PATH.parent
    subprocess.run([cc, "-std=c99", "-Wall", "-Werror", "-I", str(HEADER.parent), str(src),
                    "-L", str(lib_dir), f"-l:{_lib.LIB_PATH.name}", f"-Wl,-rpath,{lib_dir}",
                    "-o", str(exe)], check=True, capture_output=True)
    run = subprocess.run([str(exe)], capture_output=True, text=True, timeout=60)
    assert run.returncode == 0, (run.returncode, run.stderr)
    seen = {}
    for line in run.stdout.splitlines():
        s, f, v = line.split()
        seen[(s, f)] = int(v)
    for s, cls in structs.items():
        assert seen[(s, "size")] == ctypes.sizeof(cls), s
        for f, _ in cls._fields_:
            assert seen[(s, f)] == getattr(cls, f).offset, (s, f)


def test_tuning_cache_file_helpers(tmp_path, monkeypatch):
    """The autotuner's JSON cache on the host: the path follows
    $DIFFMPM_GB300_TUNING_CACHE, writes merge keys and replace the file
    whole, and an unreadable or corrupt file reads as empty."""
    from diffmpm_gb300 import engine
    path = tmp_path / "sub" / "tuning.json"
    monkeypatch.setenv("DIFFMPM_GB300_TUNING_CACHE", str(path))
    assert engine.tuning_cache_path() == path
    assert engine._read_tuning_cache(path) == {}
    a = {"block_steps": 100, "resort_every": 1, "nk_ctas": 3, "g2p_ctas": 2, "forces_lpc": 0,
         "ms_per_step": 1.2}
    engine._write_tuning_cache(path, "gpu|k1", a)
    engine._write_tuning_cache(path, "gpu|k2", dict(a, block_steps=50))
    got = engine._read_tuning_cache(path)
    assert got == {"gpu|k1": a, "gpu|k2": dict(a, block_steps=50)}
    assert [p.name for p in path.parent.iterdir()] == ["tuning.json"]   # no temporaries left
    path.write_text("{not json")
    assert engine._read_tuning_cache(path) == {}
    # the candidate set is part of every key's hash input
    assert "forces_lpc 0,1,2" in engine._TUNING_SPACE


def test_status_codes_map_to_python_exceptions(built):
    """Non-zero statuses raise MpmError naming the status and carrying the
    library's message; MPM_ERR_OUT_OF_MESH raises OutOfMeshError, which is
    also a ValueError (the reference raises ValueError for bad inputs)."""
    from diffmpm_gb300 import _lib
    lib = _lib.load()
    _lib.check(_lib.MPM_OK)
    d = _lib.MpmDesc()
    d.ndim, d.scheme = 2, 7
    d.nelements[0] = d.nelements[1] = 2
    d.el_len[0] = d.el_len[1] = 0.5
    h = ctypes.c_void_p()
    rc = lib.mpm_create(ctypes.byref(d), ctypes.byref(h))
    with pytest.raises(_lib.MpmError, match="MPM_ERR_INVALID.*scheme"):
        _lib.check(rc)
    with pytest.raises(_lib.OutOfMeshError) as e:
        _lib.check(3)
    assert isinstance(e.value, ValueError) and e.value.code == 3
    with pytest.raises(_lib.MpmError) as e:
        _lib.check_batch(lib.mpm_batch_create(None, 0, ctypes.byref(ctypes.c_void_p())))
    assert e.value.code == 1 and "at least one simulation" in str(e.value)
