"""Host-side checks that need no GPU: the C-ABI library loads and exports
every symbol the public header declares, its host-only error paths, the
synthetic atmosphere generator and column sharding (gloo, 2 ranks)."""
import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest

from mima_gb300 import atmosphere as A
from mima_gb300 import rrtmg as R
from mima_gb300.shard import column_slice

ROOT = Path(__file__).resolve().parent.parent


def header_symbols():
    text = "".join(p.read_text() for p in sorted((ROOT / "include").glob("*.h")))
    return sorted(set(re.findall(r"^(?:int|const char\*|long long)\s+(rrtmg_\w+)\(", text, re.M)))


def test_library_exports_every_declared_symbol():
    lib = R.load_library()
    syms = header_symbols()
    assert len(syms) == 22
    assert set(syms) == set(R.EXPORTED)
    for s in syms:
        assert hasattr(lib, s), s


def test_integration_guide_names_every_entry_point():
    text = (ROOT / "INTEGRATION.md").read_text()
    missing = [s for s in header_symbols() if f"`{s}" not in text and f"{s}(" not in text]
    assert not missing, missing


def test_host_only_error_paths(tmp_path):
    lib = R.load_library()
    assert lib.rrtmg_gpu_error_string(0) == b"success"
    assert b"table" in lib.rrtmg_gpu_error_string(R.RRTMG_ERR_TABLES)
    h = C.c_void_p()
    # a missing blob is reported before any CUDA call
    rc = lib.rrtmg_gpu_init(C.c_double(1004.64), str(tmp_path / "nope.bin").encode(), 0, C.byref(h))
    assert rc == R.RRTMG_ERR_TABLES and not h.value
    bad = tmp_path / "bad.bin"
    bad.write_bytes(b"RRTMGTB1" + b"\0" * 40)
    assert lib.rrtmg_gpu_init(C.c_double(1004.64), str(bad).encode(), 0, C.byref(h)) == R.RRTMG_ERR_TABLES
    assert lib.rrtmg_gpu_init(C.c_double(-1.0), b"x", 0, C.byref(h)) == R.RRTMG_ERR_ARG
    assert lib.rrtmg_gpu_set_precision(None, 0) == R.RRTMG_ERR_ARG
    assert lib.rrtmg_gpu_finalize(None) == R.RRTMG_ERR_ARG
    assert lib.rrtmg_gpu_reserve(None, 10, 40) == R.RRTMG_ERR_ARG
    # run_rrtmg entry points: defaults are host-only; a null handle is refused before any CUDA call
    p = R.run_params(lonstep=2)
    assert p.lonstep == 2 and p.dt_rad_avg == 86400 and p.solr_cnst == 1368.22
    assert lib.rrtmg_run_params_default(None) == R.RRTMG_ERR_ARG
    assert lib.rrtmg_run_c(None, C.byref(p), 8, 2, 10, 0, 0, 365, *([None] * 22)) == R.RRTMG_ERR_ARG


def test_generator_configurations():
    atm = A.config_atmosphere(0)
    assert atm.ncol == 128 * 64 and atm.nlay == 40
    assert atm.play.shape == (40, 8192) and atm.plev.shape == (41, 8192)
    assert np.all(np.diff(atm.plev, axis=0) < 0)  # surface first
    assert np.isclose(atm.plev[-1, 0], 0.1) and np.isclose(atm.plev[0, 0], 1000.0)
    assert np.all((atm.tlay >= 200.0) & (atm.tlay < 340.0))
    assert np.all((atm.h2o >= 3e-6) & (atm.h2o < 0.05))
    assert np.all((atm.coszen >= 0) & (atm.coszen < 0.5))
    a3 = A.config_atmosphere(3)
    assert a3.ncol == 256
    a2 = A.grid_atmosphere("T170", 60, 12347, 5.0, True)
    assert a2.ncol == 131072 and np.isclose(a2.plev[-1, 0], 0.01)
    # reproducible
    assert np.array_equal(A.config_atmosphere(0).tsfc, atm.tsfc)


def test_column_slices_partition():
    for n in (1, 7, 8192, 32768):
        for w in (1, 2, 3, 8):
            s = [column_slice(r, w, n) for r in range(w)]
            cover = np.concatenate([np.arange(n)[x] for x in s])
            assert np.array_equal(cover, np.arange(n))


def _shard_worker(rank, world, port, q):
    import os
    import torch
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from mima_gb300 import tables
    from oracle import oracle as orc
    orc.load(tables.ensure_blob())
    atm = A.small_atmosphere(64, 40, seed=12)
    sl = column_slice(rank, world, atm.ncol)
    part = orc.rrtmg_lw(atm.subset(np.arange(atm.ncol)[sl]), nthreads=1)["uflx"]
    t = torch.from_numpy(np.ascontiguousarray(part.T))
    sizes = [torch.zeros(1, dtype=torch.long) for _ in range(world)]
    dist.all_gather(sizes, torch.tensor([t.shape[0]]))
    out = [torch.zeros((int(s), t.shape[1]), dtype=t.dtype) for s in sizes]
    dist.all_gather(out, t)
    if rank == 0:
        q.put(torch.cat(out).numpy().T.copy())
    dist.destroy_process_group()


def test_sharded_columns_gloo_world2():
    import multiprocessing as mp
    import socket
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    ps = [ctx.Process(target=_shard_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    got = q.get(timeout=120)
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    from mima_gb300 import tables
    from oracle import oracle as orc
    orc.load(tables.ensure_blob())
    full = orc.rrtmg_lw(A.small_atmosphere(64, 40, seed=12))["uflx"]
    assert np.array_equal(got, full)


def test_bench_reference_arm_line():
    """bench.py --impl reference (the CPU restatement, no GPU) prints one JSON
    line with the contract's keys, on the same workload name as the GPU arm."""
    import json
    import subprocess
    import sys
    r = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "1", "--cpu-sample", "64", "--config", "0"],
                       capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    import bench
    assert d["impl"] == "reference" and d["metric"] == bench.METRIC and d["unit"] == bench.UNIT
    assert d["value"] > 0 and d["e2e"]["value"] == d["value"] and d["cpu_baseline"]["kind"] == "port"
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["e2e"]["d2h_bytes_per_step"] == 0
    assert d["cpu_baseline"]["cores"] >= 1 and d["cpu_baseline"]["model"]
    assert d["config"]["workload"] == bench.workload_name(0, A.config_atmosphere(0))


def test_blob_reader_rejects_inconsistent_entries(tmp_path, blob):
    """rrtmg_gpu_init refuses (RRTMG_ERR_TABLES, before any CUDA call) a blob
    whose checksum is right but one of whose entries is inconsistent: bytes
    outside the file (including an offset that wraps around), a byte count that
    is not a whole number of elements, dimensions that do not match the byte
    count, an unknown type, more than 4 dimensions."""
    import struct
    from mima_gb300 import tables
    body = Path(blob).read_bytes()[:-8]
    name, dtype, ndim = struct.unpack_from("<48sII", body, 16)
    dims = struct.unpack_from("<4I", body, 16 + 72)
    off, nb = struct.unpack_from("<QQ", body, 16 + 88)
    esz = 4 if dtype == 1 else 8
    assert ndim >= 1 and nb == esz * int(np.prod(dims[:ndim]))
    cases = {"off": ("<Q", 88, 2**64 - 8), "nb": ("<Q", 96, nb - 1), "dims": ("<I", 72, dims[0] + 1),
             "dtype": ("<I", 48, 7), "ndim": ("<I", 52, 5), "nb_past_end": ("<Q", 96, len(body) + 64)}
    lib = R.load_library()
    for case, (fmt, at, value) in cases.items():
        raw = bytearray(body)
        struct.pack_into(fmt, raw, 16 + at, value)
        p = tmp_path / f"{case}.bin"
        p.write_bytes(bytes(raw) + struct.pack("<Q", tables.blob_checksum(bytes(raw))))
        h = C.c_void_p()
        assert lib.rrtmg_gpu_init(C.c_double(1004.64), str(p).encode(), 0, C.byref(h)) == R.RRTMG_ERR_TABLES, case
        assert not h.value
    # the unpatched blob passes the reader (then needs a GPU: RRTMG_ERR_CUDA without one)
    h = C.c_void_p()
    rc = lib.rrtmg_gpu_init(C.c_double(1004.64), str(blob).encode(), 0, C.byref(h))
    assert rc != R.RRTMG_ERR_TABLES
    if h.value:
        lib.rrtmg_gpu_finalize(h)


# ---- the Python mirror's device-array wrappers against the C header ---------

class _FakeTensor:
    """Stands in for a CUDA float64 tensor: the attributes the wrappers read."""

    def __init__(self, numel, ptr, dtype="torch.float64", cuda=True, contiguous=True, index=0):
        import types
        self._n, self._p, self._c = numel, ptr, contiguous
        self.dtype, self.is_cuda, self.device = dtype, cuda, types.SimpleNamespace(index=index)

    def numel(self):
        return self._n

    def data_ptr(self):
        return self._p

    def is_contiguous(self):
        return self._c


class _RecordingLib:
    def __init__(self):
        self.calls = {}

    def __getattr__(self, name):
        def fn(*args):
            self.calls[name] = args
            return 0
        return fn


def _header_params(fn):
    text = "".join(p.read_text() for p in sorted((ROOT / "include").glob("*.h")))
    m = re.search(r"^int\s+" + fn + r"\((.*?)\);", text, re.S | re.M)
    return [re.findall(r"(\w+)\s*$", a.strip())[0] for a in m.group(1).split(",")]


def _mirror():
    r = object.__new__(R.RRTMG)
    r._h, r.device, r.lib = C.c_void_p(1), 0, _RecordingLib()
    r._check = lambda rc: None
    return r


def _ptr(a):
    return None if a is None else C.cast(a, C.c_void_p).value


def _check_positions(call, params, expect):
    """Every pointer parameter carries the fake tensor of its name, or NULL."""
    assert len(call) == len(params)
    for name, arg in zip(params, call):
        if name in expect:
            assert _ptr(arg) == expect[name], name


def test_device_wrappers_follow_the_header():
    ncol, nlay = 5, 7
    sizes = R.array_sizes(ncol, nlay)
    fake = {k: _FakeTensor(n, 0x10000 * (i + 1)) for i, (k, n) in enumerate(sorted(sizes.items()))}
    ptr = {k: t.data_ptr() for k, t in fake.items()}
    cloud_lw = ["cldfr", "taucld", "cicewp", "cliqwp", "reice", "reliq"]
    r = _mirror()
    # rrtmg_lw_dev: the LW aerosol argument is the tauaer keyword
    r.rrtmg_lw_dev(0, ncol, nlay, 0, 1, fake, fake, tauaer=fake["tauaer_lw"])
    exp = {k: ptr[k] for k in _header_params("rrtmg_lw_dev") if k in ptr and k != "tauaer"}
    # the cloud arrays, the cloud-physics sizes among them, pass through by name
    exp.update({"tauaer": ptr["tauaer_lw"]})
    _check_positions(r.lib.calls["rrtmg_lw_dev"], _header_params("rrtmg_lw_dev"), exp)
    r.rrtmg_lw_dev(0, ncol, nlay, 2, 1, fake, fake, inflglw=2, iceflglw=3, liqflglw=1)
    call, par = r.lib.calls["rrtmg_lw_dev"], _header_params("rrtmg_lw_dev")
    assert [call[par.index(k)].value for k in ("inflglw", "iceflglw", "liqflglw")] == [2, 3, 1]
    r.rrtmg_lw_dev_static(0, ncol, nlay, 0, 1, fake, fake, tauaer=None)
    exp.update({"tauaer": None, **{k: None for k in cloud_lw}})
    _check_positions(r.lib.calls["rrtmg_lw_dev_static"], _header_params("rrtmg_lw_dev_static"), exp)
    # rrtmg_sw_dev: tauaer/ssaaer/asmaer are the SW arrays of the input dict
    r.rrtmg_sw_dev(0, ncol, nlay, 0, 10, fake, fake, 1.0, 0, 1360.0)
    p = _header_params("rrtmg_sw_dev")
    exp = {k: ptr[k] for k in p if k in ptr}
    exp.update({k: None for k in cloud_lw + ["ssacld", "asmcld", "fsfcld", "ecaer"]})
    _check_positions(r.lib.calls["rrtmg_sw_dev"], p, exp)
    # SW clouds come from the cloud keyword (14-band arrays), never the input dict
    cl = {"cldfr": fake["cldfr"], "taucld": fake["taucld_sw"], "ssacld": fake["ssacld"], "asmcld": fake["asmcld"],
          "fsfcld": fake["fsfcld"], "cicewp": fake["cicewp"]}
    r.rrtmg_sw_dev(0, ncol, nlay, 1, 0, fake, fake, 1.0, 0, 1360.0, cloud=cl)
    exp.update({k: C.cast(t.data_ptr(), C.c_void_p).value for k, t in cl.items()})
    exp.update(cliqwp=None)
    _check_positions(r.lib.calls["rrtmg_sw_dev"], p, exp)
    # cloud physics: the sizes and the flags of the cloud keyword
    phys = {"cldfr": fake["cldfr"], "cicewp": fake["cicewp"], "cliqwp": fake["cliqwp"], "reice": fake["reice"],
            "reliq": fake["reliq"], "inflag": 2, "iceflag": 3, "liqflag": 1}
    r.rrtmg_sw_dev(0, ncol, nlay, 1, 0, fake, fake, 1.0, 0, 1360.0, cloud=phys)
    exp.update({k: ptr[k] for k in ("cldfr", "cicewp", "cliqwp", "reice", "reliq")})
    exp.update(taucld=None, ssacld=None, asmcld=None, fsfcld=None)
    call = r.lib.calls["rrtmg_sw_dev"]
    _check_positions(call, p, exp)
    assert [call[p.index(k)].value for k in ("inflgsw", "iceflgsw", "liqflgsw")] == [2, 3, 1]
    with pytest.raises(ValueError):  # a per-layer array is too small for the 14-band taucld
        r.rrtmg_sw_dev(0, ncol, nlay, 1, 0, fake, fake, 1.0, 0, 1360.0, cloud={**cl, "taucld": fake["cldfr"]})
    # rrtmg_step_dev
    r.rrtmg_step_dev(0, ncol, nlay, fake, fake, fake, 1.0, 0, 1360.0, idrv=1, iaer=10,
                     tauaer_lw=fake["tauaer_lw"])
    p = _header_params("rrtmg_step_dev")
    exp = {k: ptr[k] for k in p if k in ptr}
    exp.update(tauaer_lw=ptr["tauaer_lw"], tauaer_sw=ptr["tauaer"])
    _check_positions(r.lib.calls["rrtmg_step_dev"], p, exp)
    # adjoint: aerosols only as keywords; an input dict's SW aerosols are not picked up
    nx, ny = R.adjoint_shape(nlay)
    jac, cot, grad = _FakeTensor(nx * ny * ncol, 0xA0000), _FakeTensor(ny * ncol, 0xB0000), _FakeTensor(nx * ncol, 0xC0000)
    r.jacobian_dev(0, ncol, nlay, fake, jac, 1.0, 0, 1360.0)
    p = _header_params("rrtmg_jacobian_dev")
    exp = {k: ptr[k] for k in p if k in ptr and k not in ("tauaer_lw", "tauaer_sw", "ssaaer", "asmaer")}
    exp.update(tauaer_lw=None, tauaer_sw=None, ssaaer=None, asmaer=None, jac=0xA0000)
    _check_positions(r.lib.calls["rrtmg_jacobian_dev"], p, exp)
    r.vjp_dev(0, ncol, nlay, fake, cot, grad, 1.0, 0, 1360.0, iaer=10, tauaer_sw=fake["tauaer"],
              ssaaer=fake["ssaaer"], asmaer=fake["asmaer"])
    p = _header_params("rrtmg_vjp_dev")
    exp.pop("jac")
    exp.update(tauaer_sw=ptr["tauaer"], ssaaer=ptr["ssaaer"], asmaer=ptr["asmaer"], cot=0xB0000, grad=0xC0000)
    _check_positions(r.lib.calls["rrtmg_vjp_dev"], p, exp)
    # run_rrtmg_dev
    si, sj, sk = 8, 3, nlay
    rs = R.run_array_sizes(si, sj, sk)
    rfake = {k: _FakeTensor(n, 0x100000 * (i + 1)) for i, (k, n) in enumerate(sorted(rs.items()))}
    r.run_rrtmg_dev(0, R.run_params(), si, sj, sk, 0, 0, 365, rfake, rfake)
    p = _header_params("rrtmg_run_dev")
    _check_positions(r.lib.calls["rrtmg_run_dev"], p, {k: t.data_ptr() for k, t in rfake.items()})


def test_device_wrappers_refuse_wrong_tensors():
    ncol, nlay = 5, 7
    sizes = R.array_sizes(ncol, nlay)
    good = {k: _FakeTensor(n, 0x10000 * (i + 1)) for i, (k, n) in enumerate(sorted(sizes.items()))}
    r = _mirror()
    bad = {"short": _FakeTensor(sizes["play"] - 1, 0x1), "float32": _FakeTensor(sizes["play"], 0x1, dtype="torch.float32"),
           "host": _FakeTensor(sizes["play"], 0x1, cuda=False), "strided": _FakeTensor(sizes["play"], 0x1, contiguous=False),
           "other_gpu": _FakeTensor(sizes["play"], 0x1, index=1)}
    for case, t in bad.items():
        with pytest.raises(ValueError):
            r.rrtmg_lw_dev(0, ncol, nlay, 0, 0, {**good, "play": t}, good)
        assert "rrtmg_lw_dev" not in r.lib.calls, case
    with pytest.raises(ValueError, match="uflx has"):
        r.rrtmg_lw_dev(0, ncol, nlay, 0, 0, good, {**good, "uflx": _FakeTensor(sizes["uflx"] - 1, 0x2)})
    nx, ny = R.adjoint_shape(nlay)
    with pytest.raises(ValueError, match="grad has"):
        r.vjp_dev(0, ncol, nlay, good, _FakeTensor(ny * ncol, 0x3), _FakeTensor(nx * ncol - 1, 0x4), 1.0, 0, 1360.0)


def test_run_params_layout_agrees_everywhere():
    """rrtmg_run_params has one member order in the C header, the ctypes
    mirror and the Fortran bind(C) type of the integration guide, and the
    library's defaults fill the ctypes structure (a host-only call)."""
    hdr = (ROOT / "include" / "rrtmg_run.h").read_text()
    body = re.search(r"typedef struct\s*\w*\s*\{(.*?)\}\s*rrtmg_run_params;", hdr, re.S).group(1)
    body = re.sub(r"/\*.*?\*/", "", body, flags=re.S)
    c_fields = []
    for decl in body.split(";"):
        m = re.match(r"\s*(int|double)\s+(.*)$", decl.strip(), re.S)
        if m:
            c_fields += [(m.group(1), n.strip()) for n in m.group(2).split(",")]
    py_fields = [("int" if t is C.c_int else "double", n) for n, t in R.RunParams._fields_]
    assert c_fields == py_fields
    guide = (ROOT / "INTEGRATION.md").read_text()
    ftype = re.search(r"type, bind\(C\) :: rrtmg_run_params(.*?)end type", guide, re.S).group(1)
    f_fields = []
    for kind, names in re.findall(r"(integer\(c_int\)|real\(c_double\)) ::(.*?)(?=integer\(c_int\)|real\(c_double\)|$)",
                                  ftype.replace("&", " ").replace("!", "\n!"), re.S):
        names = re.sub(r"!.*", "", names)
        f_fields += [("int" if kind.startswith("integer") else "double", n.strip())
                     for n in names.split(",") if n.strip()]
    assert f_fields == c_fields
    assert C.sizeof(R.RunParams) == 10 * 4 + 22 * 8
    p = R.run_params()
    assert (p.lonstep, p.dt_rad_avg, p.co2ppmv, p.obliq, p.solr_cnst) == (1, 86400, 300.0, 23.439, 1368.22)


def test_fortran_interfaces_follow_the_header():
    """Every bind(C) interface of the integration guide lists the C entry
    point's arguments in the header's order (by name where the Fortran uses
    the header's names; by count for rrtmg_gpu_init and
    rrtmg_run_params_default)."""
    guide = (ROOT / "INTEGRATION.md").read_text()
    found = {}
    for m in re.finditer(r"function\s+(rrtmg_\w+)\s*\((.*?)\)\s*(?:&\s*)?bind\(C,\s*name=\"(\w+)\"\)", guide, re.S):
        args = [a.strip() for a in m.group(2).replace("&", " ").split(",")]
        assert m.group(1) == m.group(3)
        found[m.group(1)] = args
    assert {"rrtmg_gpu_init", "rrtmg_lw_c", "rrtmg_sw_c", "rrtmg_run_c", "rrtmg_run_params_default"} <= set(found)
    for fn, args in found.items():
        params = _header_params(fn)
        assert len(args) == len(params), fn
        if fn not in ("rrtmg_gpu_init", "rrtmg_run_params_default"):
            assert args == params, (fn, [(a, b) for a, b in zip(args, params) if a != b])


def test_fortran_dropin_calls_pass_each_argument_in_place():
    """The drop-in rrtmg_lw / rrtmg_sw of the integration guide pass every
    argument to rrtmg_lw_c / rrtmg_sw_c in its header position: each actual
    argument, stripped of its kind conversion, names the dummy it lands on
    (the handle and the optional-derivative pointers by their roles)."""
    guide = (ROOT / "INTEGRATION.md").read_text()
    roles = {"rrtmg_gpu": "h", "pd": "duflx_dt", "pdc": "duflxc_dt"}
    for fn in ("rrtmg_lw_c", "rrtmg_sw_c"):
        m = re.search(r"call rrtmg_gpu_check\(" + fn + r"\((.*?)\), \"rrtmg_", guide, re.S)
        assert m, fn
        text = m.group(1).replace("&", " ")
        args, depth, cur = [], 0, ""
        for ch in text:
            depth += (ch == "(") - (ch == ")")
            if ch == "," and depth == 0:
                args.append(cur.strip())
                cur = ""
            else:
                cur += ch
        args.append(cur.strip())
        names = []
        for a in args:
            k = re.match(r"(?:int|real)\((\w+),\s*c_\w+\)$", a)
            names.append(roles.get(a, k.group(1) if k else a))
        assert names == _header_params(fn), (fn, [(x, y) for x, y in zip(names, _header_params(fn)) if x != y])


def test_profile_summaries_state_their_commands():
    """Every committed ncu summary gives the command that made it (a command
    that runs committed files only), and every ncu command in it leaves the
    GPU clocks alone."""
    summaries = sorted((ROOT / "profiles").glob("*.md"))
    assert summaries
    for p in summaries:
        text = p.read_text()
        ncu = [ln for ln in text.splitlines() if ln.lstrip().startswith("ncu ")]
        captures = [ln for ln in ncu if not ln.lstrip().startswith("ncu -i ")]  # -i reads a saved report
        assert captures, p.name
        assert all("--clock-control none" in ln for ln in captures), p.name
        assert "python" in text and "..." not in "\n".join(ln for ln in text.splitlines() if "python " in ln), p.name
        assert "_work" not in text, p.name
