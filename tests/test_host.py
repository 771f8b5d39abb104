"""CPU: the C ABI loads and exports every declared symbol, host-side logic
(generators, --nb resolution, argument checks, the CLI's parser) and the
integer/float helpers shared by host and device code."""
import re
import subprocess
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent


def declared_functions(header: Path):
    text = re.sub(r"/\*.*?\*/", "", header.read_text(), flags=re.S)
    return sorted(set(re.findall(r"\b(rmq_[a-z0-9_]+)\s*\(", text)))


def test_every_declared_symbol_is_exported(native):
    names = declared_functions(ROOT / "include" / "rmq.h")
    assert "rmq_build" in names and "rmq_query" in names and "rmq_free" in names
    missing = [n for n in names if not hasattr(native, n)]
    assert not missing, missing
    from rtxrmq_gb300._native import SIGNATURES
    assert sorted(SIGNATURES) == names


def test_version_and_error_string(native):
    assert b"sm_103a" in native.rmq_version()
    import rtxrmq_gb300 as R
    with pytest.raises(R.RMQError) as e:
        R.bs_from_nb(0, 5)
    assert e.value.code == -1 and "n=0" in str(e.value)


@pytest.mark.parametrize("n,nb,bs", [(10**8, 512, 195312), (10**8, 8192, 12207), (100, 1000, 1),
                                     (100, 3, 33), (7, 7, 1)])
def test_bs_from_nb_matches_reference_cli(native, n, nb, bs):
    """src/tools.h:129-132: nb = min(n, nb); bs = n / nb."""
    import rtxrmq_gb300 as R
    assert R.bs_from_nb(n, nb) == bs


def test_null_handle_calls_fail_cleanly(native):
    import ctypes as C
    assert native.rmq_query(None, None, 1, None, None, None) == -1
    assert native.rmq_free(None) == 0
    h = C.c_void_p()
    assert native.rmq_build(None, 10, 0, None, C.byref(h)) == -1
    assert native.rmq_build(None, 0, 0, None, C.byref(h)) == -1
    assert native.rmq_query_scan(None, 10, None, 1, None, None, None) == -1


def test_generators_deterministic_and_prefix_stable(native):
    import rtxrmq_gb300 as R
    a = R.gen_values_uniform(100_000, 1321)
    assert a.dtype == np.float32 and a.min() >= 0.0 and a.max() < 1.0
    np.testing.assert_array_equal(a, R.gen_values_uniform(100_000, 1321))
    np.testing.assert_array_equal(a[:777], R.gen_values_uniform(777, 1321))
    q1 = R.gen_queries(5000, 10**6, -3, 9)
    np.testing.assert_array_equal(q1[:100], R.gen_queries(100, 10**6, -3, 9))
    # 24-bit resolution: values are multiples of 2^-24
    assert np.all((a * 2**24) == np.floor(a * 2**24))


@pytest.mark.parametrize("lr", [-1, -2, -3, -4, -5, 1, 32, 1024])
def test_query_modes(native, lr):
    import rtxrmq_gb300 as R
    n = 10**6
    Q = R.gen_queries(200_000, n, lr, 1321)
    l, r = Q[:, 0].astype(np.int64), Q[:, 1].astype(np.int64)
    assert (l >= 0).all() and (l <= r).all() and (r < n).all()
    ln = r - l + 1
    if lr > 0:
        assert (ln == lr).all()
    elif lr == -1:
        assert abs(ln.mean() / (n / 2) - 1) < 0.01
    else:
        mu = {-2: 0.6 * np.log(n), -3: 0.3 * np.log(n), -4: np.log(n // 256),
              -5: np.log(n // 32768)}[lr]
        # median of a lognormal is exp(mu)
        assert abs(np.median(ln) / np.exp(mu) - 1) < 0.02
        assert abs(np.log(ln).std() - 0.3) < 0.02


def test_config1_mean_length(native):
    """Config n=1e6, q=2^20, lengths round(lognormal(0.3 ln n, 0.3)): mean
    exp(mu + sigma^2/2) = 66.0 (the reference's truncating generator with
    scale floor(n^0.3) gives 65.4)."""
    import rtxrmq_gb300 as R
    Q = R.gen_queries(1 << 20, 10**6, -3, 1321)
    expect = np.exp(0.3 * np.log(1e6) + 0.3**2 / 2)
    assert abs((Q[:, 1] - Q[:, 0] + 1).mean() - expect) < 0.3


def test_value_generators(native):
    import rtxrmq_gb300 as R
    z = R.gen_values_normal(200_000, 5)
    assert abs(z.mean()) < 0.01 and abs(z.std() - 1) < 0.01
    k = R.gen_values_int(200_000, 256, 5)
    assert set(np.unique(k)) == set(range(256))


HELPER_TEST = r"""
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>
#include <cmath>
#include "common.cuh"
using namespace rmq;
static unsigned long long rng = 88172645463325252ull;
static unsigned next() { rng ^= rng << 13; rng ^= rng >> 7; rng ^= rng << 17; return (unsigned)rng; }
static float f(unsigned b) { float x; std::memcpy(&x, &b, 4); return x; }
int main() {
  std::vector<unsigned> ds = {1,2,3,4,5,6,7,8,9,10,11,12,13,31,32,33,63,64,65,100,127,128,129,
     1000,1023,1024,1025,4095,4096,4097,12207,32767,32768,32769,65535,65536,195312,1000000,
     (1u<<30)-1, 1u<<30, (1u<<30)+1, 0x7fffffffu};
  for (int i = 0; i < 2000; ++i) ds.push_back(1 + next() % 0x7fffffffu);
  for (int i = 0; i < 2000; ++i) ds.push_back(1 + next() % 70000u);
  for (unsigned d : ds) {
    Div31 D = make_div31(d);
    std::vector<unsigned> xs = {0u, 1u, d - 1, d, d + 1, 0x7fffffffu, 0x7ffffffeu};
    for (unsigned k = 1; k < 40; ++k) { unsigned long long m = (unsigned long long)k * d;
      if (m < 0x80000000ull) { xs.push_back((unsigned)m); xs.push_back((unsigned)m - 1); } }
    for (unsigned long long m = d; m < 0x80000000ull; m *= 3) { xs.push_back((unsigned)m - 1); xs.push_back((unsigned)m); }
    for (int i = 0; i < 2000; ++i) xs.push_back(next() & 0x7fffffffu);
    for (unsigned x : xs) if (x <= 0x7fffffffu && div31(x, D) != x / d) {
      std::printf("div31 mismatch d=%u x=%u got %u\n", d, x, div31(x, D)); return 1; }
  }
  // fkey: order preserving for float <, -0 == +0, NaN above +inf, funkey inverse
  std::vector<unsigned> bs = {0u, 0x80000000u, 0x7f800000u, 0xff800000u, 1u, 0x80000001u,
                              0x3f800000u, 0xbf800000u, 0x00800000u, 0x80800000u, 0x7f7fffffu, 0xff7fffffu};
  for (int i = 0; i < 4000; ++i) { unsigned b = next(); if (!std::isnan(f(b))) bs.push_back(b); }
  for (unsigned a : bs) {
    if (funkey(fkey(a), a == 0x80000000u) != a) { std::printf("funkey %08x\n", a); return 1; }
    for (unsigned b : bs) {
      bool lt = f(a) < f(b), eq = f(a) == f(b);
      if (lt != (fkey(a) < fkey(b)) || eq != (fkey(a) == fkey(b))) {
        std::printf("fkey order %08x %08x\n", a, b); return 1; }
    }
  }
  unsigned nanb[] = {0x7fc00000u, 0xffc00000u, 0x7f800001u, 0xffffffffu};
  for (unsigned nb : nanb) if (fkey(nb) != 0xffffffffu || fkey(nb) <= fkey(0x7f800000u)) { std::printf("nan\n"); return 1; }
  for (unsigned k = 1; k < 33; ++k) { unsigned x = (k == 32) ? 0xffffffffu : (1u << k) - 1;
    if (ilog2(x) != (int)std::floor(std::log2((double)x))) { std::printf("ilog2 %u\n", x); return 1; } }
  std::printf("ok\n");
  return 0;
}
"""


def test_device_helpers_on_host(tmp_path, native):
    """common.cuh compiled for the host: exact magic division for every
    31-bit dividend class, order-preserving float keys, ilog2."""
    src = tmp_path / "t.cpp"
    src.write_text(HELPER_TEST)
    exe = tmp_path / "t"
    cuda_inc = Path("/usr/local/cuda/include")
    r = subprocess.run(["g++", "-O2", "-std=c++17", f"-I{ROOT / 'rtxrmq_gb300' / 'csrc'}",
                        f"-I{cuda_inc}", str(src), "-o", str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and "ok" in r.stdout, r.stdout + r.stderr


LANE_TEST = r"""
#include <cstdio>
#include <vector>
#include "lane_min.cuh"
using namespace rmq;
static unsigned long long rng = 0x9E3779B97F4A7C15ull;
static unsigned next() { rng ^= rng << 13; rng ^= rng >> 7; rng ^= rng << 17; return (unsigned)rng; }
// definition: among b[0 .. nvalid), the smallest key, leftmost among equal
// keys; no valid value: the largest key at position 0
template <uint32_t MODE> static bool check(const uint32_t (&b)[4], uint32_t nvalid) {
  uint32_t ek = 0xffffffffu, ep = 0u, en = 0u;
  for (uint32_t k = 0; k < nvalid; ++k) {
    const uint32_t kk = key_of(b[k], MODE);
    if (k == 0 || kk < ek) { ek = kk; ep = k; en = negzero_of(b[k], MODE); }
  }
  uint32_t key, info;
  lane_best4<MODE>(b, nvalid, key, info);
  const uint32_t want = ep | (en << 2);
  if (key != ek || (nvalid > 0 && info != want) || (nvalid == 0 && (info & 3u) != 0u)) {
    std::printf("mode %u nvalid %u: %08x %08x %08x %08x -> key %08x info %u, want %08x %u\n", MODE,
                nvalid, b[0], b[1], b[2], b[3], key, info, ek, want);
    return false;
  }
  return true;
}
int main() {
  // special values: +-0, +-inf, NaNs of both signs and payloads, subnormals,
  // the extremes, small integers (ties), and random bits
  std::vector<unsigned> pool = {0u, 0x80000000u, 0x7f800000u, 0xff800000u, 0x7fc00000u,
      0xffc00000u, 0x7f800001u, 0xffbfffffu, 1u, 0x80000001u, 0x007fffffu, 0x807fffffu,
      0x3f800000u, 0xbf800000u, 0x7f7fffffu, 0xff7fffffu, 0x40000000u, 0xc0000000u,
      0x80000000u, 0x00000000u, 0x7fffffffu, 0xffffffffu};
  for (int i = 0; i < 24; ++i) pool.push_back(next());
  long n = 0;
  for (int it = 0; it < 120000; ++it) {
    uint32_t b[4];
    for (int k = 0; k < 4; ++k) b[k] = (next() & 3) ? pool[next() % pool.size()] : next();
    for (uint32_t nv = 0; nv <= 4; ++nv) {
      if (!check<kFloatMin>(b, nv) || !check<kFloatMax>(b, nv) || !check<kIntMin>(b, nv) ||
          !check<kIntMax>(b, nv)) return 1;
      ++n;
    }
  }
  std::printf("ok %ld\n", n);
  return 0;
}
"""


def test_lane_minimum_matches_key_order(tmp_path, native):
    """lane_best4 (the per-lane step of the light index's micro-block minima),
    compiled for the host: for four values with any number valid, in every
    key mode, the key and position of the smallest key, leftmost among equal
    keys. Covers +-0 ties, NaNs of either sign, subnormals and infinities,
    where the float modes' IEEE minimum / maximum path must agree with the
    key order."""
    src = tmp_path / "lane.cpp"
    src.write_text(LANE_TEST)
    exe = tmp_path / "lane"
    r = subprocess.run(["g++", "-O2", "-std=c++17", f"-I{ROOT / 'rtxrmq_gb300' / 'csrc'}",
                        "-I/usr/local/cuda/include", str(src), "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and r.stdout.startswith("ok"), r.stdout + r.stderr


CLI = ROOT / "rtxrmq_gb300" / "_lib" / "rtxrmq"


@pytest.mark.parametrize("args,code", [([], 1), (["0", "10", "1", "5"], 1), (["100", "10", "101", "5"], 1),
                                       (["1000", "10", "-1", "0"], 2), (["1000", "10", "-1", "1"], 2),
                                       (["1000", "10", "-1", "101"], 2), (["1000", "10", "-1", "3"], 2)])
def test_cli_argument_errors(native, args, code):
    """Argument errors and algorithms outside this engine exit before any
    CUDA call (src/tools.h:76-95 checks)."""
    r = subprocess.run([str(CLI), *args], capture_output=True, text=True, timeout=60)
    assert r.returncode == code, r.stdout + r.stderr


def test_ragged_workload_shapes(native):
    from rtxrmq_gb300 import workloads as W
    w = W.ragged(narrays=64, umin=8, umax=12, total_q=20000, seed=3)
    assert w.lengths.min() >= 256 and w.lengths.max() <= 4096
    assert (w.starts % 4 == 0).all() and w.total_q == 20000 == int(w.qcounts.sum())
    assert w.span >= int((w.starts + w.lengths).max())
    for s, c, n in zip(w.qstarts, w.qcounts, w.lengths):
        q = w.queries[s:s + c]
        assert (q[:, 0] >= 0).all() and (q[:, 0] <= q[:, 1]).all() and (q[:, 1] < n).all()
    # queries proportional to length
    assert abs(np.corrcoef(w.qcounts, w.lengths)[0, 1] - 1) < 1e-3
    d = W.differentiable_rows(nrows=8, lmin=1000, lmax=2000, q_per_row=100, seed=4)
    assert d.span == int(d.lengths.sum()) and (d.qcounts == 100).all()
    assert abs(float(d.values.mean())) < 0.1


FAKE_NVML = r"""
int nvmlInit_v2(void) { return 0; }
int nvmlShutdown(void) { return 0; }
int nvmlDeviceGetHandleByIndex_v2(unsigned i, void **d) { *d = (void *)0x1234; return i == 0 ? 0 : 2; }
int nvmlDeviceGetHandleByPciBusId_v2(const char *b, void **d) { *d = (void *)0x1234; return 0; }
int nvmlDeviceGetPowerUsage(void *d, unsigned *mw) { *mw = 250000u; return d == (void *)0x1234 ? 0 : 1; }
"""


def test_power_sampler_against_fake_nvml(native, tmp_path, monkeypatch):
    """rmq_power_begin / end (the role of GPUPowerBegin / GPUPowerEnd,
    common/nvmlPower.cpp) against a fake NVML that reports 250 W: the table
    has the reference's columns, energy integrates power over time."""
    import time

    from rtxrmq_gb300.power import PowerSampler
    src = tmp_path / "fake_nvml.c"
    src.write_text(FAKE_NVML)
    so = tmp_path / "libfake_nvml.so"
    r = subprocess.run(["gcc", "-shared", "-fPIC", "-o", str(so), str(src)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    monkeypatch.setenv("RTXRMQ_NVML_LIBRARY", str(so))
    table = tmp_path / "power.dat"
    with PowerSampler(0, sample_ms=20, path=str(table)) as p:
        assert p.available
        assert native.rmq_power_begin(0, 20, 0, None) == -1  # one sampler at a time
        time.sleep(0.3)
    assert abs(p.avg_watts - 250.0) < 1e-9
    assert abs(p.energy_joules - 250.0 * p.seconds) < 1e-6 and 0.2 < p.seconds < 1.0
    lines = table.read_text().splitlines()
    assert lines[0].split() == ["#timestep", "power", "acc-energy", "avg-power", "dt", "acc-time"]
    rows = [list(map(float, ln.split())) for ln in lines[1:]]
    assert len(rows) >= 5 and all(row[1] == 250.0 for row in rows)
    assert abs(rows[-1][2] - p.energy_joules) < 1e-3
    assert native.rmq_power_end(0, None, None, None) == -1  # not running
    monkeypatch.setenv("RTXRMQ_NVML_LIBRARY", str(tmp_path / "missing.so"))
    with PowerSampler(0) as q:
        assert not q.available and q.status == -5


def test_bench_and_entry_compile():
    """bench.py and __graft_entry__.py are valid Python (the GPU legs are
    only exercised on a GPU; this catches syntax errors on the CPU)."""
    import py_compile
    root = Path(__file__).resolve().parent.parent
    for f in ("bench.py", "__graft_entry__.py"):
        py_compile.compile(str(root / f), doraise=True)


def _bench_module():
    import importlib.util
    spec = importlib.util.spec_from_file_location("bench", ROOT / "bench.py")
    bench = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(bench)
    return bench


def test_bench_reference_arm(oracle_lib):
    """`bench.py --impl reference` (the reference's CPU comparator, HRMQ
    restated) prints one JSON line with the contract's keys and the GPU
    arm's config, and never imports this package (its inputs come from
    bench.py's own numpy generators)."""
    import json
    import subprocess
    import sys
    root = Path(__file__).resolve().parent.parent
    code = ("import runpy, sys; sys.argv = ['bench.py'] + sys.argv[1:]; "
            "runpy.run_path('bench.py', run_name='__main__'); "
            "assert not [m for m in sys.modules if m.startswith('rtxrmq_gb300')], 'package imported'")
    r = subprocess.run([sys.executable, "-c", code, "--impl", "reference", "--n", "1000000",
                        "--q", "100000", "--steps", "3", "--warmup", "3"],
                       cwd=root, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    line = json.loads([x for x in r.stdout.splitlines() if x.startswith("{")][-1])
    assert line["impl"] == "reference" and line["value"] > 0 and line["unit"] == "RMQ/s"
    assert line["cpu_baseline"]["kind"] == "port" and line["cpu_baseline"]["cores"] >= 1
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["steps"] == 3
    bench = _bench_module()
    assert line["config"] == bench.headline_config(1000000, 100000, -1)[2]
    assert line["metric"] == "RMQ/s n=1000000 q=100000 lr=-1 (values+indices)"


def test_bench_traffic_profile_digest(tmp_path):
    """roofline.traffic comes from the committed ncu summary only while the
    query kernel's sources are the ones it was captured from: a summary
    with another digest (or none) gives no bytes and says why."""
    bench = _bench_module()
    digest = bench.query_sources_digest()
    assert len(digest) == 64 and digest == bench.query_sources_digest()
    prof = tmp_path / "p.md"
    bench.TRAFFIC_PROFILE = prof
    prof.write_text(f"x\ntraffic_bytes_per_query: 15.5\ntraffic_bs: 16384\n"
                    f"traffic_sources_sha256: {digest}\n")
    b, info = bench.profiled_traffic(1000)
    assert b == 15500.0 and info["bs"] == 16384 and "stale" not in info
    prof.write_text("traffic_bytes_per_query: 15.5\ntraffic_sources_sha256: 00\n")
    b, info = bench.profiled_traffic(1000)
    assert b is None and "changed" in info["stale"]
    prof.unlink()
    assert bench.profiled_traffic(1000) == (None, {"source": None, "stale": "no traffic profile"})


def test_bench_query_generators():
    """bench.py's numpy inputs: queries in range with the reference's length
    modes (fixed, uniform, lognormal 0.6 / 0.3 ln n), deterministic in the
    seed; values in [0, 1) and tie-heavy integers."""
    import math
    bench = _bench_module()
    n, q = 10**6, 200_000
    for lr in (-1, -2, -3, 1, 1024, n):
        Q = bench.np_queries(q, n, lr, 7)
        assert Q.dtype == np.int32 and Q.shape == (q, 2)
        ln = Q[:, 1].astype(np.int64) - Q[:, 0] + 1
        assert (Q[:, 0] >= 0).all() and (ln >= 1).all() and (Q[:, 1] < n).all()
        if lr > 0:
            assert (ln == lr).all()
        elif lr == -1:
            assert abs(ln.mean() / (n / 2) - 1) < 0.01
        else:
            mu = {-2: 0.6, -3: 0.3}[lr] * math.log(n)
            assert abs(np.log(ln).mean() - mu) < 0.01
        assert np.array_equal(Q, bench.np_queries(q, n, lr, 7))
    A = bench.np_values_uniform(n, 1)
    assert A.dtype == np.float32 and A.min() >= 0 and A.max() < 1
    T = bench.np_values_int(n, 256, 1)
    assert set(np.unique(T)) == set(float(x) for x in range(256))


def test_bench_accounting():
    """Algorithmic bytes from the kernel's counts: 16 B per query plus 32 B
    per per-element entry and per scanned sector; skipped lookups against
    the un-pruned two per query."""
    bench = _bench_module()
    st = {"first_probe": 90, "second_probe": 6, "full": 2, "micro_scan": 0, "block_edge": 0,
          "warp_scan": 1, "entries": 10, "table_words": 300, "scan_sectors": 3, "invalid": 1}
    acc = bench.stats_bytes(st, 100)
    assert acc["alg_bytes"] == 100 * 16 + 32 * 13
    assert acc["unpruned_alg_bytes"] == 100 * 80
    assert acc["entries_per_query"] == 10 / 99
    assert abs(acc["entry_lookups_skipped"] - (1 - 10 / 198)) < 1e-12
    assert abs(sum(acc["settled"].values()) - 1.0) < 1e-12


def test_normal_build_reports_not_checked(native):
    """rmq_checked_violations answers RMQ_ENOTSUP outside the checked build."""
    import ctypes as C
    cnt = C.c_int64(-1)
    assert native.rmq_checked_violations(C.byref(cnt)) == -5  # RMQ_ENOTSUP
    assert cnt.value == 0


def test_batch_argument_types(native):
    """The batched form refuses values that are not float32 and queries that
    are not int32 [q, 2] before anything reaches the device."""
    import torch

    from rtxrmq_gb300 import batch as B
    with pytest.raises(TypeError):
        B._vals(torch.zeros(4, dtype=torch.float64))
    with pytest.raises(TypeError):
        B._queries(torch.zeros((4, 2), dtype=torch.int64))
    with pytest.raises(TypeError):
        B._queries(torch.zeros((4, 3), dtype=torch.int32))
    # an int32 plan takes int32 values only (on the CPU a value tensor of the
    # right type passes the type check and is refused as not on the device)
    with pytest.raises(ValueError):
        B._vals(torch.zeros(4, dtype=torch.int32), int32=True)
    with pytest.raises(TypeError):
        B._vals(torch.zeros(4, dtype=torch.float32), int32=True)
    with pytest.raises(TypeError):
        B._vals(torch.zeros(4, dtype=torch.int32))


def test_batch_plan_flags(native):
    """RMQBatch(op, dtype, light) maps to rmq_batch_create_ex's flags
    (include/rmq.h's RMQ_BUILD_* bits), from strings or torch dtypes."""
    import torch

    from rtxrmq_gb300 import batch as B
    from rtxrmq_gb300._native import RMQ_BUILD_INT32, RMQ_BUILD_LIGHT, RMQ_BUILD_MAX
    assert B.plan_flags() == 0
    assert B.plan_flags("max") == RMQ_BUILD_MAX
    assert B.plan_flags(dtype="int32") == B.plan_flags(dtype=torch.int32) == RMQ_BUILD_INT32
    assert B.plan_flags("max", torch.int32, True) == RMQ_BUILD_MAX | RMQ_BUILD_INT32 | RMQ_BUILD_LIGHT
    assert B.plan_flags(dtype=torch.float32, light=True) == RMQ_BUILD_LIGHT
    header = (Path(__file__).resolve().parent.parent / "include" / "rmq.h").read_text()
    for name, val in (("RMQ_BUILD_MAX", RMQ_BUILD_MAX), ("RMQ_BUILD_INT32", RMQ_BUILD_INT32),
                      ("RMQ_BUILD_LIGHT", RMQ_BUILD_LIGHT)):
        assert re.search(rf"#define {name}\s+{val}u", header), name
    with pytest.raises(ValueError):
        B.plan_flags("median")
    with pytest.raises(TypeError):
        B.plan_flags(dtype="float64")


def test_random_parity_cases_are_valid(native):
    """The seeded random configurations of the GPU parity tests produce
    in-range queries and consistent layouts (checked here without a GPU)."""
    import sys
    sys.path.insert(0, str(Path(__file__).resolve().parent))
    import test_gpu_batch as TB
    import test_gpu_parity as TP
    for seed in range(64):
        n, bs, dtype, op, micro, off, A, Q = TP.random_case(seed)
        assert 1 <= bs <= n and len(A) == n and 0 <= off < 4
        assert A.dtype == np.dtype(dtype) and op in ("min", "max")
        assert (Q[:, 0] >= 0).all() and (Q[:, 0] <= Q[:, 1]).all() and (Q[:, 1] < n).all()
    for seed in range(24):
        starts, lengths, qstarts, qcounts, V, Q, bucket_bs = TB.random_batch(seed)
        assert (starts >= 0).all() and (starts + lengths <= len(V)).all() and len(bucket_bs) == 32
        assert (qstarts[1:] >= qstarts[:-1] + qcounts[:-1]).all()
        assert (qstarts + qcounts <= len(Q)).all()
        for n, q0, c in zip(lengths, qstarts, qcounts):
            if n and c:
                q = Q[q0:q0 + c]
                assert (q[:, 0] >= 0).all() and (q[:, 0] <= q[:, 1]).all() and (q[:, 1] < n).all()
