"""C-ABI checks that need no GPU: the library loads, exports exactly the
symbols include/gbnde.h declares, the ctypes mirrors have the C layout, and
calls without a device fail with an error code instead of crashing."""
import ctypes as C
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "gbnde.h")


def _declared():
    txt = re.sub(r"/\*.*?\*/", "", open(HEADER).read(), flags=re.S)  # drop comments
    pat = r"^\s*(?:const\s+)?(?:int|void|size_t|long\s+long|char)\s*\**\s*(gbnde_[a-z_]+)\s*\("
    return sorted(set(re.findall(pat, txt, flags=re.M)))


def test_exports_every_declared_symbol(lib):
    out = subprocess.run(["nm", "-D", "--defined-only", lib._name], capture_output=True, text=True).stdout
    exported = set(re.findall(r" T (gbnde_[a-z_]+)", out))
    declared = set(_declared())
    assert declared, "no declarations parsed"
    assert declared <= exported, f"missing: {declared - exported}"
    assert exported <= declared, f"undeclared exports: {exported - declared}"


def test_ctypes_layout_matches_c(tmp_path):
    import gbnde._lib as L
    src = tmp_path / "sz.c"
    src.write_text(
        '#include <stdio.h>\n#include <stddef.h>\n#include "gbnde.h"\n'
        "int main(void){printf(\"%zu %zu %zu %zu %zu %zu %zu %zu\\n\", sizeof(gbnde_mlp_desc),"
        " sizeof(gbnde_solve_desc), sizeof(gbnde_stats), offsetof(gbnde_solve_desc, saveat),"
        " offsetof(gbnde_stats, retcode), offsetof(gbnde_stats, t_final),"
        " offsetof(gbnde_stats, fwd_path), offsetof(gbnde_stats, adj_path));return 0;}\n")
    exe = tmp_path / "sz"
    subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    vals = [int(v) for v in subprocess.run([str(exe)], capture_output=True, text=True).stdout.split()]
    assert vals == [C.sizeof(L.MlpDesc), C.sizeof(L.SolveDesc), C.sizeof(L.Stats),
                    L.SolveDesc.saveat.offset, L.Stats.retcode.offset, L.Stats.t_final.offset,
                    L.Stats.fwd_path.offset, L.Stats.adj_path.offset]


def test_strerror_and_errors_without_device(lib):
    import gbnde._lib as L
    assert lib.gbnde_strerror(L.ERR_INVALID) == b"invalid argument"
    assert lib.gbnde_strerror(12345) == b"unknown error"
    h = C.c_void_p()
    assert lib.gbnde_create(None, None, 0, 0) == L.ERR_INVALID
    d = L.MlpDesc()
    d.nlayers = 0
    assert lib.gbnde_create(C.byref(h), C.byref(d), 0, 0) == L.ERR_INVALID
    d.nlayers = 1
    d.dims[0], d.dims[1] = 4, 5          # output dim != state dim
    assert lib.gbnde_create(C.byref(h), C.byref(d), 0, 0) == L.ERR_INVALID
    d.dims[1] = 4
    d.act[0] = 9
    assert lib.gbnde_create(C.byref(h), C.byref(d), 0, 0) == L.ERR_INVALID
    assert lib.gbnde_forward_steps(None, None, None, 0) == 0
    assert lib.gbnde_nparams(None) == 0
    lib.gbnde_destroy(None)


def test_layer_api_validation():
    import numpy as np
    import gbnde
    m = gbnde.Chain(gbnde.cube(), gbnde.Dense(2, 50, "tanh"), gbnde.Dense(50, 2))
    assert m.nparams() == 2 * 50 + 50 + 50 * 2 + 2 == 252
    assert m.cube_input and m.dims == [2, 50, 2]
    with pytest.raises(ValueError):
        gbnde.Dense(2, 3, "relu")
    with pytest.raises(ValueError):
        gbnde.Chain(gbnde.Dense(2, 3), gbnde.Dense(4, 2))
    with pytest.raises(TypeError):
        gbnde.NeuralODE(m, (0.0, 1.0), object(), saveat=[0, 1])
    # no saveat: every step is saved (the reference's save_everystep default)
    assert gbnde.NeuralODE(m, (0.0, 1.0), gbnde.Tsit5()).save_everystep
    assert not gbnde.NeuralODE(m, (0.0, 1.0), gbnde.Tsit5(), saveat=[0.0, 1.0]).save_everystep
    node = gbnde.NeuralODE(m, (0.0, 1.0), gbnde.Tsit5(), saveat=0.1)
    assert len(node.saveat) == 11 and node.saveat[0] == 0.0 and abs(node.saveat[-1] - 1.0) < 1e-12
    node = gbnde.NeuralODE(m, (0.0, 1.0), gbnde.Tsit5(), save_everystep=False, save_start=False)
    assert node.saveat == [1.0]
    p = m.init_params(np.random.default_rng(0))
    assert p.dtype == np.float32 and p.size == 252
    # bias entries are zero, weights bounded by the Glorot limit
    assert np.all(p[100:150] == 0) and np.abs(p[:100]).max() <= np.sqrt(6 / 52)


def test_tuning_knobs_reject_bad_arguments(lib):
    import gbnde._lib as L
    assert lib.gbnde_set_grid_cap(None, 0) == L.ERR_INVALID
    assert lib.gbnde_set_stage_memory(None, 0) == L.ERR_INVALID
