"""CPU-side checks of the C ABI library: it loads without a GPU, exports every
entry point include/nxb_gb300.h declares, validates arguments before touching
the device, and its struct layouts match the reference's."""
import ctypes
import re
import subprocess
from pathlib import Path

import pytest

import nexusbvh_gb300 as nxb

ROOT = Path(__file__).resolve().parent.parent
HEADER = ROOT / "include" / "nxb_gb300.h"


def declared_functions():
    text = re.sub(r"/\*.*?\*/", "", HEADER.read_text(), flags=re.S)
    return sorted(set(re.findall(r"\b(nxb_[a-z0-9_]+)\s*\(", text)))


@pytest.fixture(scope="module")
def lib():
    from nexusbvh_gb300 import _build
    _build.build_cuda()
    return nxb.load()


def test_library_exports_every_declared_symbol(lib):
    names = declared_functions()
    assert len(names) >= 20
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    out = subprocess.run(["nm", "-D", "--defined-only", str(nxb.lib_path())], capture_output=True, text=True).stdout
    for n in names:
        assert re.search(rf"\bT {n}$", out, flags=re.M), n


def test_status_strings_and_version(lib):
    for code, name in nxb.STATUS_NAMES.items():
        assert lib.nxb_status_string(code).decode() == name
    assert "sm_103a" in nxb.version()


def test_argument_checks_need_no_device(lib):
    out = nxb.CBVH8()
    c = nxb.BuildConfig().to_c()
    assert lib.nxb_build_bvh8(None, 1, 10, ctypes.byref(c), None, ctypes.byref(out), None) == 1
    assert lib.nxb_build_bvh8(16, 1, 0, ctypes.byref(c), None, ctypes.byref(out), None) == 1
    assert lib.nxb_build_bvh8(16, 7, 10, ctypes.byref(c), None, ctypes.byref(out), None) == 1
    assert lib.nxb_build_bvh8(16, 1, 1 << 31, ctypes.byref(c), None, ctypes.byref(out), None) == 2
    bad = nxb.BuildConfig(search_radius=5).to_c()
    assert lib.nxb_build_bvh8(16, 1, 10, ctypes.byref(bad), None, ctypes.byref(out), None) == 2
    assert lib.nxb_build_bvh8(16, 1, 10, ctypes.byref(c), None, None, None) == 1


def test_workspace_requirement_needs_no_device(lib):
    """nxb_build_async rejects a short workspace before it touches the
    device: a BVH8 build needs the queried size, a build that stops at the
    BVH2 needs 64 bytes per primitive less (no child-pair records)."""
    n = 100_000
    c = nxb.BuildConfig().to_c()
    s = nxb.CSizes()
    assert lib.nxb_query_build_sizes(n, ctypes.byref(c), ctypes.byref(s)) == 0
    fake = 1 << 20  # 256-byte aligned addresses the call never dereferences before this check
    short_bvh8 = s.workspace_bytes - 1
    assert lib.nxb_build_async(fake, 1, n, ctypes.byref(c), fake, short_bvh8, fake, fake, fake, fake, None) == 5
    short_bvh2 = s.workspace_bytes - 64 * n - 1
    assert lib.nxb_build_async(fake, 1, n, ctypes.byref(c), fake, short_bvh2, fake, None, None, fake, None) == 5


def test_workspace_sizes(lib):
    s = nxb.CSizes()
    for bits, kb in ((30, 4), (63, 8)):
        cfg = nxb.BuildConfig(prioritize_speed=bits == 30).to_c()
        n = 12_582_912
        assert lib.nxb_query_build_sizes(n, ctypes.byref(cfg), ctypes.byref(s)) == 0
        assert s.bvh2_node_count == 2 * n - 1
        assert s.bvh8_node_capacity == (4 * n - 1 + 6) // 7
        # keys x2, values x2, parent slots, BVH8 work slots, H-PLOC cluster
        # records, child-pair records, look-back
        assert s.workspace_bytes >= n * (2 * kb + 8 + 4 + 8 + 32 + 64)
        assert s.workspace_bytes < n * (2 * kb + 8 + 4 + 8 + 32 + 64 + 8)
    assert lib.nxb_query_build_sizes(0, None, ctypes.byref(s)) == 1
    # NXB_BUILD_VALIDATE belongs to the plain calls only
    v = nxb.BuildConfig(validate=True).to_c()
    assert v.flags == nxb.NXB_BUILD_VALIDATE
    assert lib.nxb_query_build_sizes(1000, ctypes.byref(v), ctypes.byref(s)) == 2


def test_validator_argument_checks_need_no_device(lib):
    def seg(b):
        return (b + 255) // 256 * 256
    n = 1000
    need2 = lib.nxb_validate_bvh2_scratch_bytes(n)
    # links, parent counts, leaf counts, one word per pointer-jumping round
    assert need2 == seg(8 * (2 * n - 1)) + seg(4 * (2 * n - 1)) + seg(4 * n) + seg(4 * 32)
    assert lib.nxb_validate_bvh2_scratch_bytes(0) == 0
    assert lib.nxb_validate_bvh2_scratch_bytes(1 << 31) == 0
    m = 300
    need8 = lib.nxb_validate_bvh8_scratch_bytes(m, n)
    assert need8 == seg(8 * m) + 3 * seg(4 * m) + seg(24 * m) + seg(4 * n) + seg(4 * 32)
    assert lib.nxb_validate_bvh8_scratch_bytes(0, n) == 0 and lib.nxb_validate_bvh8_scratch_bytes(m, 0) == 0
    # every call below is rejected before anything is enqueued
    assert lib.nxb_validate_bvh2(None, n, 0, 16, 16, need2, None) == 1
    assert lib.nxb_validate_bvh2(16, n, 2 * n - 1, 16, 16, need2, None) == 1
    assert lib.nxb_validate_bvh2(16, n, 0, 16, 16, need2 - 1, None) == 1
    assert lib.nxb_validate_bvh2(16, 0, 0, 16, 16, need2, None) == 1
    assert lib.nxb_validate_bvh2(16, n, 0, None, 16, need2, None) == 1
    assert lib.nxb_validate_bvh8(16, m, 16, n, 16, 7, 16, 16, need8, None) == 1
    assert lib.nxb_validate_bvh8(16, m, 16, n, None, 1, 16, 16, need8, None) == 1
    assert lib.nxb_validate_bvh8(16, m, 16, n, 16, 1, 16, 16, need8 - 1, None) == 1
    assert lib.nxb_validate_bvh8(16, 0, 16, n, 16, 1, 16, 16, need8, None) == 1


def test_struct_layouts():
    assert ctypes.sizeof(nxb.CAABB) == 24
    assert ctypes.sizeof(nxb.CBVH2) == 40 and ctypes.sizeof(nxb.CBVH8) == 56
    assert nxb.CBVH8.prim_idx.offset == 16 and nxb.CBVH8.bounds.offset == 28
    assert nxb.BVH2_NODE_DTYPE.itemsize == 32 and nxb.BVH8_NODE_DTYPE.itemsize == 80
    assert nxb.BVH8_NODE_DTYPE.fields["meta"][1] == 24 and nxb.BVH8_NODE_DTYPE.fields["qhi"][1] == 56


def test_cpp_facade_compiles(tmp_path):
    src = tmp_path / "use.cpp"
    src.write_text(
        '#include "NXB/BVHBuilder.h"\n'
        "static_assert(sizeof(NXB::BVH2::Node) == 32, \"\");\n"
        "static_assert(sizeof(NXB::BVH8::Node) == 80, \"\");\n"
        "static_assert(sizeof(NXB::BVH8::NodeExplicit) == 80, \"\");\n"
        "static_assert(sizeof(NXB::Triangle) == 36, \"\");\n"
        "static_assert(sizeof(NXB::BVH2) == 40 && sizeof(NXB::BVH8) == 56, \"\");\n"
        "NXB::BVH8 f(NXB::Triangle* t, uint32_t n) {\n"
        "  NXB::BuildConfig c; c.prioritizeSpeed = true;\n"
        "  NXB::BVHBuildMetrics m;\n"
        "  return NXB::BuildBVH8<NXB::Triangle>(t, n, c, &m);\n"
        "}\n"
        "NXB::BVH2 g(NXB::AABB* b, uint32_t n) { return NXB::BuildBVH2(b, n); }\n"
        '#include "NXB/BatchBuilder.h"\n'
        "NXB::BVH8 h(NXB::Triangle* t, const std::vector<uint32_t>& counts) {\n"
        "  NXB::BuildConfig c; c.prioritizeSpeed = true; c.useAuction = true;\n"
        "  NXB::BatchBuilder<NXB::Triangle> b(counts, c);\n"
        "  b.Autotune(t); b.Build(t);\n"
        "  return b.MeshBVH8(0);\n"
        "}\n"
        "NXB::BVH8 s(const NXB::Triangle* t, uint32_t n) {\n"
        "  NXB::BuildServer srv(1ull << 30, 2);\n"
        "  uint64_t k = srv.Submit(t, n, false);\n"
        "  nxb_server_result info{};\n"
        "  NXB::BVH8 r = srv.Wait(k, &info);\n"
        "  srv.Release(k);\n"
        "  return r;\n"
        "}\n")
    proc = subprocess.run(["g++", "-std=c++17", "-fsyntax-only", f"-I{ROOT / 'include'}", "-I/usr/local/cuda/include",
                           str(src)], capture_output=True, text=True)
    assert proc.returncode == 0, proc.stderr


def test_batch_argument_checks_need_no_device(lib):
    import numpy as np
    h = ctypes.c_void_p()
    c30 = nxb.BuildConfig(prioritize_speed=True).to_c()
    c63 = nxb.BuildConfig(prioritize_speed=False).to_c()
    ok = np.array([0, 10, 20], dtype=np.uint32)
    dec = np.array([0, 10, 5], dtype=np.uint32)
    first = np.array([3, 10, 20], dtype=np.uint32)
    assert lib.nxb_batch_create(1, ok.ctypes.data, 2, None, ctypes.byref(h)) == 2      # default = 63-bit
    assert lib.nxb_batch_create(1, ok.ctypes.data, 2, ctypes.byref(c63), ctypes.byref(h)) == 2
    assert lib.nxb_batch_create(1, dec.ctypes.data, 2, ctypes.byref(c30), ctypes.byref(h)) == 1
    assert lib.nxb_batch_create(1, first.ctypes.data, 2, ctypes.byref(c30), ctypes.byref(h)) == 1
    assert lib.nxb_batch_create(1, ok.ctypes.data, 0, ctypes.byref(c30), ctypes.byref(h)) == 1
    assert lib.nxb_batch_create(5, ok.ctypes.data, 2, ctypes.byref(c30), ctypes.byref(h)) == 1
    assert lib.nxb_batch_create(1, None, 2, ctypes.byref(c30), ctypes.byref(h)) == 1
    bad_r = nxb.BuildConfig(prioritize_speed=True, search_radius=5).to_c()
    assert lib.nxb_batch_create(1, ok.ctypes.data, 2, ctypes.byref(bad_r), ctypes.byref(h)) == 2
    big = np.array([0, 1 << 30], dtype=np.uint32)
    assert lib.nxb_batch_create(1, big.ctypes.data, 1, ctypes.byref(c30), ctypes.byref(h)) == 2
    assert lib.nxb_batch_destroy(None) == 1
    assert lib.nxb_batch_build(None, None, None, None) == 1


def test_server_argument_checks_need_no_device(lib):
    h = ctypes.c_void_p()
    bad = nxb.CServerConfig(0, 0, 0, 0, 2)
    assert lib.nxb_server_create(ctypes.byref(bad), ctypes.byref(h)) == 2
    many = nxb.CServerConfig(0, 65, 0, 0, 0)
    assert lib.nxb_server_create(ctypes.byref(many), ctypes.byref(h)) == 2
    assert lib.nxb_server_create(None, None) == 1
    t = ctypes.c_uint64()
    assert lib.nxb_server_submit(None, None, 0, 1, 10, None, ctypes.byref(t)) == 1
    assert lib.nxb_server_wait(None, 1, None) == 1
    assert lib.nxb_server_release(None, 1) == 1
    assert lib.nxb_server_destroy(None) == 1
    assert ctypes.sizeof(nxb.CServerResult) == 96 and ctypes.sizeof(nxb.CServerStats) == 64


def test_validator_wrappers_check_tensors():
    torch = pytest.importorskip("torch")
    cpu = torch.zeros(64, dtype=torch.uint8)
    with pytest.raises(ValueError):
        nxb.validate_bvh2(cpu, 1)
    with pytest.raises(ValueError):
        nxb.validate_bvh8(cpu, 1, torch.zeros(1, dtype=torch.int32), torch.zeros((1, 9), dtype=torch.float32))


def test_every_cuda_source_is_built():
    from nexusbvh_gb300 import _build
    on_disk = sorted(p.name for p in (Path(nxb.__file__).parent / "csrc").glob("*.cu"))
    assert sorted(_build.CUDA_SOURCES) == on_disk


def test_check_report_lengths_match_the_header():
    hdr = (Path(nxb.__file__).parent.parent / "include" / "nxb_gb300.h").read_text()
    n2 = int(re.search(r"#define NXB_BVH2_CHECK_FIELDS (\d+)", hdr).group(1))
    n8 = int(re.search(r"#define NXB_BVH8_CHECK_FIELDS (\d+)", hdr).group(1))
    assert n2 == len(nxb.BVH2_CHECK_FIELDS) and n8 == len(nxb.BVH8_CHECK_FIELDS)
    assert nxb.BVH2_CHECK_FIELDS[-1] == nxb.BVH8_CHECK_FIELDS[-1] == "errors"
