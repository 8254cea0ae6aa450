"""Host-side logic and the C ABI library, without a GPU."""
import ctypes
import os
import re

import numpy as np
import pytest
import scipy.sparse as sps

import oracle
from pq_testutil import ROOT, dok_from, golden, lattice


@pytest.fixture(scope="session")
def native():
    import build_native
    build_native.build()
    from piqmc import _native
    return _native.lib()


def _header_symbols():
    text = open(os.path.join(ROOT, "include", "piqmc_gb300.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(pq_\w+)\s*\(", text)))


def test_library_exports_every_header_symbol(native):
    syms = _header_symbols()
    assert len(syms) >= 20
    lib = ctypes.CDLL(os.path.join(ROOT, "pathintegral-qmc_gb300", "piqmc", "_native", "libpiqmc_gb300.so"))
    missing = [s for s in syms if not hasattr(lib, s)]
    assert not missing, missing
    from piqmc import _native
    assert set(_native.SIGNATURES) >= set(syms)
    assert native.pq_version() >= 1
    assert native.pq_strerror(2) == b"index outside [0, nspins)"


def test_generate_neighbors_golden_and_random(native):
    from piqmc import tools
    g = golden("neighbors_5node")
    J = dok_from(g["rows"], g["cols"], g["vals"], 5)
    np.testing.assert_array_equal(tools.GenerateNeighbors(5, J, 4), g["nbs"])
    rng = np.random.default_rng(3)
    for trial in range(5):
        n = 30
        A = sps.random(n, n, density=0.08, random_state=trial, format="dok")
        for i in range(0, n, 3):
            A[i, i] = rng.normal()
        deg = np.zeros(n, int)
        for (a, b) in A.keys():
            deg[a] += 1
            if a != b:
                deg[b] += 1
        m = int(deg.max())
        np.testing.assert_array_equal(tools.GenerateNeighbors(n, A, m), oracle.generate_neighbors(n, A, m))
        with pytest.raises(IndexError):
            tools.GenerateNeighbors(n, A, m - 1)


def test_generate_neighbors_savepath(native, tmp_path):
    from piqmc import tools
    J = lattice(4, True, np.random.default_rng(0))
    p = str(tmp_path / "nbs.npy")
    nbs = tools.GenerateNeighbors(16, J, 4, savepath=p)
    np.testing.assert_array_equal(np.load(p), nbs)


def test_bits_spins():
    from piqmc import tools
    a = np.array([0., 1., 0., 1., 0., 1., 0., 1., 0., 1.])
    b = tools.bits2spins(a)
    assert np.all(b == [1, -1, 1, -1, 1, -1, 1, -1, 1, -1])
    assert np.all(tools.spins2bits(b) == a)


def test_jperp_matches_oracle(native):
    from piqmc.reforder import jperp_schedule
    for P, T in [(20, 0.05), (5, 0.01), (32, 1.7), (2, 0.3)]:
        s = np.linspace(3.0, 1e-8, 57)
        np.testing.assert_array_equal(jperp_schedule(s, P, T), oracle.jperp(s, P, T))
    with pytest.raises(ZeroDivisionError):
        jperp_schedule(np.ones(3), 4, 0.0)


def test_libc_peek_does_not_advance_and_skip_does(native):
    from piqmc.reforder import libc_peek, libc_skip
    oracle.libc_srand(1234)
    a = libc_peek(1000)
    b = oracle.libc_rand(1000)
    np.testing.assert_array_equal(a, b)
    oracle.libc_srand(99)
    peek = libc_peek(50)
    libc_skip(20)
    np.testing.assert_array_equal(oracle.libc_rand(30), peek[20:])


def _problem(nbs):
    from piqmc import fast
    return fast.Problem(nbs, on_device=False)


@pytest.mark.parametrize("L,periodic,fields", [(8, True, False), (7, True, True), (6, False, True), (16, True, False)])
def test_problem_classes_are_independent_sets(native, L, periodic, fields):
    from piqmc import tools
    g = np.random.default_rng(L)
    J = lattice(L, periodic, g, fields=(lambda r: r.normal()) if fields else None)
    nbs = tools.GenerateNeighbors(L * L, J, 5 if fields else 4)
    p = _problem(nbs)
    n = L * L
    assert sorted(p.perm.tolist()) == sorted(set(p.perm.tolist())) and len(p.perm) == n
    assert np.all(p.inv[p.perm] == np.arange(n))
    assert p.nclass <= 32 and p.nclass * p.class_stride == p.nslots
    cls = p.perm // p.class_stride
    assert np.all(p.perm % p.class_stride < p.class_size[cls])
    # independence: no coupling inside a class
    for (a, b) in J.keys():
        if a != b:
            assert cls[a] != cls[b]
    # SoA tables: every coupling of spin i appears (device slots) with its FP32 value
    for i in range(n):
        row = [(int(p.nbr_host[m, p.perm[i]]), float(p.cpl_host[m, p.perm[i]])) for m in range(p.nbr_host.shape[0])
               if p.cpl_host[m, p.perm[i]] != 0.0]
        want = [(int(p.perm[int(j)]), float(np.float32(v))) for j, v in nbs[i] if int(j) != i and v != 0.0]
        assert row == want
    # FP64 CSR reproduces the classical energy
    s = np.where(g.random(n) < 0.5, -1.0, 1.0)
    sd = np.zeros(p.nslots)
    sd[p.perm] = s
    E = 0.0
    for r in range(p.nslots):
        for e in range(p.csr_ptr[r], p.csr_ptr[r + 1]):
            c = p.csr_col[e]
            E += p.csr_val[e] * sd[r] * (1.0 if c == r else sd[c])
    assert abs(-E - oracle.classical_energy(s, J)) < 1e-10


def test_greedy_colouring(native):
    from piqmc import _native, tools
    J = lattice(5, True, np.random.default_rng(1))
    nbs = tools.GenerateNeighbors(25, J, 4)
    idx = np.ascontiguousarray(np.trunc(nbs[:, :, 0]).astype(np.int32))
    jv = np.ascontiguousarray(nbs[:, :, 1].astype(np.float32))
    col = np.empty(25, np.int32)
    nc = native.pq_color_graph(25, 4, idx.ctypes.data, jv.ctypes.data, col.ctypes.data)
    assert nc >= 3
    for (a, b) in J.keys():
        assert col[a] != col[b]


def _colour(native, L, periodic, seed):
    from piqmc import tools
    J = lattice(L, periodic, np.random.default_rng(seed))
    n = L * L
    nbs = tools.GenerateNeighbors(n, J, 4)
    idx = np.ascontiguousarray(np.trunc(nbs[:, :, 0]).astype(np.int32))
    jv = np.ascontiguousarray(nbs[:, :, 1].astype(np.float32))
    col = np.empty(n, np.int32)
    nc = native.pq_color_graph(n, 4, idx.ctypes.data, jv.ctypes.data, col.ctypes.data)
    for (a, b) in J.keys():
        assert a == b or col[a] != col[b]
    assert set(col.tolist()) == set(range(nc))
    return nc, col, J


@pytest.mark.parametrize("L", [5, 9, 15, 33])
def test_colouring_odd_torus_uses_three_colours(native, L):
    """Greedy in spin order needs 4 colours on an odd periodic lattice; DSatur finds 3."""
    nc, _, _ = _colour(native, L, True, L)
    assert nc == 3


@pytest.mark.parametrize("L,periodic", [(8, True), (16, True), (7, False), (10, False)])
def test_colouring_bipartite_keeps_greedy(native, L, periodic):
    nc, col, J = _colour(native, L, periodic, L)
    assert nc == 2
    # greedy in spin order on a connected bipartite lattice: colour = checkerboard from spin 0
    x, y = np.arange(L * L) % L, np.arange(L * L) // L
    assert np.array_equal(col, (x + y) % 2)


def test_class_layout_even_and_odd_lattices(native):
    """Balanced two-colourings keep subclasses classes per colour; a small third colour gets one class."""
    from piqmc import fast, tools
    for L, want_classes in ((80, 14), (32, 16), (8, 16)):
        J = lattice(L, True, np.random.default_rng(L))
        p = fast.Problem(tools.GenerateNeighbors(L * L, J, 4), on_device=False)
        assert p.nclass == want_classes
    J = lattice(33, True, np.random.default_rng(3))
    p = fast.Problem(tools.GenerateNeighbors(33 * 33, J, 4), on_device=False)
    assert p.ncolors == 3 and p.nclass <= 18
    assert p.nslots <= 1.15 * 33 * 33


GENERATORS = {
    "ising2d_5": lambda t, rs: t.Generate2DIsingInstance(5, rs),
    "ising2d_2": lambda t, rs: t.Generate2DIsingInstance(2, rs),
    "lattice_4x5_periodic": lambda t, rs: t.Generate2DLattice(4, 5, rs, 1),
    "lattice_4x5_open": lambda t, rs: t.Generate2DLattice(4, 5, rs, 0),
    "kblock_5x6_k2": lambda t, rs: t.GenerateKblockLattice(5, 6, rs, 2),
    "kblock_4x4_k1": lambda t, rs: t.GenerateKblockLattice(4, 4, rs, 1),
}


@pytest.mark.parametrize("name", sorted(GENERATORS))
def test_instance_generators_match_reference(name):
    """Key order, values and the rng state left behind, against the compiled reference's outputs."""
    from piqmc import tools
    g = golden("generators")
    rs = np.random.RandomState(int(g[name + "_seed"]))
    J = GENERATORS[name](tools, rs)
    items = list(J.items())
    np.testing.assert_array_equal([k[0] for k, _ in items], g[name + "_rows"])
    np.testing.assert_array_equal([k[1] for k, _ in items], g[name + "_cols"])
    np.testing.assert_array_equal([v for _, v in items], g[name + "_vals"])
    assert rs.randint(2 ** 31) == g[name + "_next_rng"]


def test_instance_file_and_neighbor_cache_round_trip(tmp_path):
    from piqmc import tools
    J = tools.Generate2DIsingInstance(6, np.random.RandomState(3))
    path = tmp_path / "inst.txt"
    with open(path, "w") as f:
        for (i, j), v in J.items():
            f.write("%d %d %.17g\n" % (i + 1, j + 1, v))
    K = tools.LoadIsingInstance(str(path))
    assert list(K.keys()) == list(J.keys())
    assert all(K[k] == v for k, v in J.items())
    nbs = tools.GenerateNeighbors(36, K, 4, str(tmp_path / "nbs.npy"))
    np.testing.assert_array_equal(tools.LoadNeighbors(str(tmp_path / "nbs.npy")), nbs)
    with pytest.raises(ValueError):
        bad = tmp_path / "bad.txt"
        bad.write_text("0 1 0.5\n")
        tools.LoadIsingInstance(str(bad))


def test_autotune_plan_balances_the_batch():
    """The batch planner keeps the efficient tile where it can and splits the items that would outlast the rest."""
    from piqmc import autotune
    slots = 2432
    small = {(1, 8, 1): 3.0e11, (1, 1, 1): 1.0e11, (8, 1, 1): 0.5e11}
    big = {(1, 8, 1): 3.0e11, (2, 1, 1): 2.5e11, (8, 1, 1): 2.0e11}
    # many small instances and one large one: the large one's (1, 8) item alone would take
    # 2048*64*8 / 1.23e8 = 8.5 ms per step against ~1 ms for the whole batch's load
    shapes = [(64, 16, 8)] * 200 + [(2048, 64, 8)]
    tiles, pred = autotune.plan(shapes, [small] * 200 + [big], slots)
    assert tiles[:200] == [(1, 8, 1)] * 200
    assert tiles[200] == (8, 1, 1)
    w8 = big[(8, 1, 1)] / slots
    total = (200 * 64 * 16 * 8 / (small[(1, 8, 1)] / slots) + 2048 * 64 * 8 / w8) / slots
    assert pred == pytest.approx(max(total, 2048 * 64 / (8 * w8)))
    # a GPU full of equal small instances keeps the most efficient tile
    tiles, _ = autotune.plan([(64, 16, 8)] * 5000, [small] * 5000, slots)
    assert set(tiles) == {(1, 8, 1)}
    # tiles with more replicas than the instance has are never chosen
    tiles, _ = autotune.plan([(64, 16, 1)], [small], slots)
    assert tiles == [(8, 1, 1)] or tiles == [(1, 1, 1)]
    # a lane-pair tile that shortens the critical item wins for it
    pairs = dict(big)
    pairs[(8, 1, 2)] = 3.5e11
    tiles, _ = autotune.plan(shapes, [small] * 200 + [pairs], slots)
    assert tiles[200] == (8, 1, 2)


def test_pack_tasks_invariants():
    """Every item lands in exactly one task; a task holds one kind (warps per item, lanes per
    site, compiled sweep), at most WARPS // gwarps items and at most the shared-memory budget;
    tasks come longest item first."""
    from piqmc import batch
    g = np.random.default_rng(5)
    items = []
    for k in range(3000):
        gw = int(g.choice([1, 2, 4, 8]))
        kind = (gw, int(g.choice([1, 2])), int(g.choice([0, 1, 16, 20, 32, 64])))
        smem = int(g.integers(1, batch.SMEM_TASK_BUDGET // 2))
        items.append((float(g.exponential(1.0)), kind, smem, k))
    tasks = batch.pack_tasks(items)
    seen = [it[3] for _, lst in tasks for it in lst]
    assert sorted(seen) == list(range(len(items)))
    for kind, lst in tasks:
        assert all(it[1] == kind for it in lst)
        assert 1 <= len(lst) <= batch.WARPS // kind[0]
        assert sum(batch._align(it[2]) for it in lst) <= batch.SMEM_TASK_BUDGET
    longest = [max(it[0] for it in lst) for _, lst in tasks]
    assert longest == sorted(longest, reverse=True)
    assert batch.pack_tasks([]) == []


def test_tile_normalisation_and_sweep_variants():
    from piqmc import batch

    class Pb:
        maxdeg = 4
    pb = Pb()
    assert batch.normalise_tile((2, 4), pb, 20) == (2, 4, 1)
    assert batch.normalise_tile((2, 4, 2), pb, 20) == (2, 4, 1)      # lane pairs need P = 64
    assert batch.normalise_tile((2, 4, 2), pb, 64) == (2, 4, 2)
    pb.maxdeg = 6
    assert batch.normalise_tile((1, 1, 2), pb, 64) == (1, 1, 1)      # and four couplings
    for bad in ((3, 1), (1, 0), (1, 1, 3)):
        with pytest.raises(ValueError):
            batch.normalise_tile(bad, pb, 20)
    assert [batch.sweep_variant(P) for P in (1, 16, 20, 31, 32, 33, 64)] == [0, 16, 20, 0, 32, 1, 64]


def test_autotune_cache_round_trip(tmp_path, monkeypatch):
    """Rate tables persist as JSON keyed "gwarps,rpc,lanes"; older "gwarps,rpc" keys load as lanes 1."""
    import json
    from piqmc import autotune
    path = tmp_path / "tune.json"
    path.write_text(json.dumps({"GPU|64|16|4|8": {"1,8": 3.0e11, "2,1,2": 2.5e11}}))
    monkeypatch.setenv("PIQMC_TUNE_CACHE", str(path))
    monkeypatch.setattr(autotune, "_cache", {})
    monkeypatch.setattr(autotune, "_loaded", False)
    assert autotune.table() == {"GPU|64|16|4|8": {(1, 8, 1): 3.0e11, (2, 1, 2): 2.5e11}}
    autotune._cache["GPU|128|20|4|8"] = {(8, 1, 1): 1.0e11}
    autotune._save()
    monkeypatch.setattr(autotune, "_cache", {})
    monkeypatch.setattr(autotune, "_loaded", False)
    tab = autotune.table()
    assert tab["GPU|128|20|4|8"] == {(8, 1, 1): 1.0e11}
    assert tab["GPU|64|16|4|8"][(1, 8, 1)] == 3.0e11
    # an unreadable cache is ignored
    path.write_text("{not json")
    monkeypatch.setattr(autotune, "_cache", {})
    monkeypatch.setattr(autotune, "_loaded", False)
    assert autotune.table() == {}


def test_product_has_no_fallback_and_no_oracle(monkeypatch, tmp_path):
    """The package never reaches the oracle or working files, a missing library raises, and a
    compute call without a CUDA device raises instead of running anywhere else."""
    pkg = os.path.join(ROOT, "pathintegral-qmc_gb300")
    pat = re.compile(r"^\s*(import|from)\s+(oracle|_work)\b|['\"/](oracle|_work)/", re.M)
    for base, _, files in os.walk(pkg):
        for f in files:
            if f.endswith((".py", ".cu", ".cuh", ".cpp", ".h")):
                text = open(os.path.join(base, f)).read()
                assert not pat.search(text), os.path.join(base, f)
    from piqmc import _native
    monkeypatch.setattr(_native, "_lib", None)
    monkeypatch.setattr(_native, "LIB_PATH", str(tmp_path / "missing.so"))
    with pytest.raises(_native.NativeLibraryMissing):
        _native.lib()
    monkeypatch.undo()
    import torch
    if not torch.cuda.is_available():
        from piqmc import qmc
        g = np.random.default_rng(0)
        nbs = oracle.generate_neighbors(16, lattice(4, True, g), 4)
        with pytest.raises(_native.PiqmcError):
            qmc.QuantumAnneal(np.linspace(1, 0.1, 3), 1, 4, 0.1, 16, np.ones((16, 4)), nbs,
                              np.random.RandomState(0))


def test_integration_bindings_match_the_header():
    """Every ctypes argtypes list written out in INTEGRATION.md has one entry per parameter of the
    header's declaration, of the matching kind (V pointer, I int, L int64_t, F float)."""
    doc = open(os.path.join(ROOT, "INTEGRATION.md")).read()
    header = re.sub(r"/\*.*?\*/", "", open(os.path.join(ROOT, "include", "piqmc_gb300.h")).read(), flags=re.S)
    bound = re.findall(r"lib\.(pq_\w+)\.argtypes = \[([^\]]*)\]", doc)
    assert len(bound) >= 4
    for name, items in bound:
        decl = re.search(r"\b%s\s*\(([^)]*)\)\s*;" % name, header)
        assert decl, name
        params = [p.strip() for p in decl.group(1).split(",") if p.strip() and p.strip() != "void"]
        want = []
        for p in params:
            t = p.rsplit(None, 1)[0] if "*" not in p else "*"
            want.append("V" if "*" in p else {"int": "I", "int64_t": "L", "float": "F"}[t])
        got = [x.strip() for x in items.split(",")]
        assert got == want, (name, got, want)


def test_ctypes_signatures_match_the_header():
    """The package's ctypes table binds every header entry point with one argument per C
    parameter of the matching kind and the declared return type."""
    import ctypes
    from piqmc import _native
    header = re.sub(r"/\*.*?\*/", "", open(os.path.join(ROOT, "include", "piqmc_gb300.h")).read(), flags=re.S)
    decls = {m.group(2): (m.group(1).strip(), m.group(3))
             for m in re.finditer(r"([\w\s\*]+?)\b(pq_\w+)\s*\(([^)]*)\)\s*;", header)}
    kinds = {"int": ctypes.c_int, "int64_t": ctypes.c_int64, "uint32_t": ctypes.c_uint32,
             "uint64_t": ctypes.c_uint64, "float": ctypes.c_float, "double": ctypes.c_double}
    assert set(decls) == set(_native.SIGNATURES), set(decls) ^ set(_native.SIGNATURES)
    for name, (ret, plist) in decls.items():
        res, args = _native.SIGNATURES[name]
        params = [p.strip() for p in plist.split(",") if p.strip() and p.strip() != "void"]
        assert len(args) == len(params), name
        for p, a in zip(params, args):
            if "*" in p:
                assert a is ctypes.c_void_p or issubclass(a, ctypes._Pointer), (name, p, a)
            else:
                assert a is kinds[p.rsplit(None, 1)[0].replace("const ", "")], (name, p, a)
        ret = ret.split()[-1]
        want = {"int": ctypes.c_int, "int64_t": ctypes.c_int64, "char*": ctypes.c_char_p}.get(ret)
        if ret.endswith("*"):
            want = ctypes.c_char_p
        assert res is want, (name, ret, res)


def test_struct_layouts_match_the_header(tmp_path):
    """Sizes and field offsets of the header's structs (compiled with gcc) against the ctypes
    structures and numpy dtypes the package fills."""
    import ctypes
    import subprocess
    from piqmc import _native, batch
    fields = {
        "pq_fast_params": [f for f, _ in _native.FastParams._fields_],
        "pq_batch_run": [f for f, _ in _native.BatchRun._fields_],
        "pq_batch_inst": ["tab_off", "field_off", "csize_off", "jperp_off", "n", "P", "maxdeg", "nclass", "stride",
                          "key0", "key1", "pad_"],
        "pq_batch_item": list(batch.ITEM_DTYPE.names),
        "pq_batch_task": list(batch.TASK_DTYPE.names),
    }
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "piqmc_gb300.h"', "int main(void) {"]
    for s, fs in fields.items():
        lines.append('printf("%s %%zu\\n", sizeof(%s));' % (s, s))
        for f in fs:
            lines.append('printf("%s.%s %%zu\\n", offsetof(%s, %s));' % (s, f, s, f))
    lines.append("return 0; }")
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.check_call(["gcc", "-std=c11", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)])
    got = dict(line.split() for line in subprocess.check_output([str(exe)]).decode().split("\n") if line)
    got = {k: int(v) for k, v in got.items()}
    for cls, s in ((_native.FastParams, "pq_fast_params"), (_native.BatchRun, "pq_batch_run")):
        assert ctypes.sizeof(cls) == got[s], s
        for f, _ in cls._fields_:
            assert getattr(cls, f).offset == got["%s.%s" % (s, f)], (s, f)
    for dt, s in ((batch.INST_DTYPE, "pq_batch_inst"), (batch.ITEM_DTYPE, "pq_batch_item"),
                  (batch.TASK_DTYPE, "pq_batch_task")):
        assert dt.itemsize == got[s], s
        c_fields = fields[s]
        for name, cf in zip(dt.names, c_fields):
            assert dt.fields[name][1] == got["%s.%s" % (s, cf)], (s, name, cf)


def test_documented_python_api_exists():
    """Every ``module.name`` the Python examples in INTEGRATION.md and README.md use exists in
    the package (file citations such as piqmc/qmc.pyx are not API references)."""
    import importlib
    text = open(os.path.join(ROOT, "INTEGRATION.md")).read() + open(os.path.join(ROOT, "README.md")).read()
    mods = ("qmc", "sa", "tools", "fast", "batch", "autotune", "dense", "learned", "reforder", "tensor")
    refs = set()
    for block in re.findall(r"```python\n(.*?)```", text, re.S):
        refs.update(re.findall(r"(?<![/\w])(%s)\.([A-Za-z_]\w*)(?!\w*:\d)" % "|".join(mods), block))
    refs = {(m, a) for m, a in refs if a != "pyx"}
    assert len(refs) >= 10
    for m, a in sorted(refs):
        assert hasattr(importlib.import_module("piqmc." + m), a), "%s.%s" % (m, a)
