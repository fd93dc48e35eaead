"""The C++ facade (include/NXB/*.h) run end to end: a caller written like the
reference's own test program (NexusBVH Test/src/Main.cpp:69-72, which calls
BenchmarkBuild(NXB::BuildBVH8<NXB::Triangle>, ...)) is compiled against the
facade, linked to libnxb_gb300.so and run.  Its BVH2 (NXB::ToHost) and BVH8
must equal the trees the C ABI builds from Python for the same triangles, and
its validated build (BuildConfig::validate) must pass the device validator."""
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

import nexusbvh_gb300 as nxb
from nexusbvh_gb300 import _build, scenes
from tests import stages as S

pytestmark = pytest.mark.gpu

ROOT = Path(__file__).resolve().parent.parent

CALLER = r"""
#include <cstdio>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "NXB/BVHBuilder.h"

static bool write_file(const char* path, const void* data, size_t bytes) {
    FILE* f = std::fopen(path, "wb");
    if (!f) return false;
    bool ok = std::fwrite(data, 1, bytes, f) == bytes;
    return std::fclose(f) == 0 && ok;
}

int main(int argc, char** argv) {
    if (argc != 3) return 2;
    FILE* f = std::fopen(argv[1], "rb");
    if (!f) return 3;
    std::vector<NXB::Triangle> tris;
    NXB::Triangle t;
    while (std::fread(&t, sizeof(t), 1, f) == 1) tris.push_back(t);
    std::fclose(f);
    const uint32_t n = (uint32_t)tris.size();
    NXB::Triangle* d = nullptr;
    if (cudaMalloc(&d, n * sizeof(NXB::Triangle)) != cudaSuccess) return 4;
    if (cudaMemcpy(d, tris.data(), n * sizeof(NXB::Triangle), cudaMemcpyHostToDevice) != cudaSuccess) return 5;

    // the reference test program's call
    NXB::BuildConfig cfg;
    NXB::BVHBuildMetrics m = NXB::BenchmarkBuild(NXB::BuildBVH8<NXB::Triangle>, 2, 3, d, n, cfg);

    // a validated BVH8 build, checked once more through the C ABI validator
    NXB::BuildConfig vcfg;
    vcfg.validate = true;
    NXB::BVH8 b8 = NXB::BuildBVH8<NXB::Triangle>(d, n, vcfg);
    size_t scratch_bytes = nxb_validate_bvh8_scratch_bytes(b8.nodeCount, n);
    void* scratch = nullptr;
    uint64_t* d_rep = nullptr;
    uint64_t rep[NXB_BVH8_CHECK_FIELDS] = {};
    if (cudaMalloc(&scratch, scratch_bytes) != cudaSuccess) return 6;
    if (cudaMalloc(&d_rep, sizeof(rep)) != cudaSuccess) return 7;
    if (nxb_validate_bvh8(reinterpret_cast<const nxb_bvh8_node*>(b8.nodes), b8.nodeCount, b8.primIdx, n, d,
                          NXB_PRIM_TRIANGLE, d_rep, scratch, scratch_bytes, nullptr) != NXB_OK)
        return 8;
    if (cudaMemcpy(rep, d_rep, sizeof(rep), cudaMemcpyDeviceToHost) != cudaSuccess) return 9;

    std::vector<unsigned char> nodes8((size_t)b8.nodeCount * 80);
    std::vector<uint32_t> prim(n);
    if (cudaMemcpy(nodes8.data(), b8.nodes, nodes8.size(), cudaMemcpyDeviceToHost) != cudaSuccess) return 10;
    if (cudaMemcpy(prim.data(), b8.primIdx, 4ull * n, cudaMemcpyDeviceToHost) != cudaSuccess) return 11;

    NXB::BVH2 b2 = NXB::BuildBVH2<NXB::Triangle>(d, n, cfg);
    NXB::BVH2 h2 = NXB::ToHost(b2);
    std::string out(argv[2]);
    if (!write_file((out + ".bvh2").c_str(), h2.nodes, (size_t)h2.nodeCount * 32)) return 12;
    if (!write_file((out + ".bvh8").c_str(), nodes8.data(), nodes8.size())) return 13;
    if (!write_file((out + ".prim").c_str(), prim.data(), 4ull * n)) return 14;
    std::printf("result %u %u %llu %.6f %.6f\n", b8.nodeCount, h2.nodeCount,
                (unsigned long long)rep[NXB_BVH8_CHECK_FIELDS - 1], m.totalTime, m.bvh8Cost);
    NXB::FreeHostBVH(h2);
    NXB::FreeDeviceBVH(b2);
    NXB::FreeDeviceBVH(b8);
    cudaFree(scratch);
    cudaFree(d_rep);
    cudaFree(d);
    return 0;
}
"""


def test_cpp_caller_through_the_facade(gpu, orc, tmp_path):
    if shutil.which("g++") is None:
        pytest.skip("no host C++ compiler")
    src = tmp_path / "caller.cpp"
    src.write_text(CALLER)
    exe = tmp_path / "caller"
    libdir = nxb.lib_path().parent
    r = subprocess.run([_build.nvcc(), "-std=c++17", "-O2", "-cudart", "shared", str(src), "-o", str(exe),
                        "-I", str(ROOT / "include"), "-L", str(libdir), "-lnxb_gb300",
                        "-Xlinker", f"-rpath,{libdir}"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr

    prims = scenes.clustered(20_000, seed=41)
    n = prims.shape[0]
    inp = tmp_path / "tris.bin"
    inp.write_bytes(np.ascontiguousarray(prims, dtype=np.float32).tobytes())
    out = tmp_path / "out"
    run = subprocess.run([str(exe), str(inp), str(out)], capture_output=True, text=True, timeout=120)
    assert run.returncode == 0, (run.returncode, run.stdout, run.stderr)
    line = [ln for ln in run.stdout.splitlines() if ln.startswith("result ")][-1].split()
    nodes8, nodes2, errors, total_ms, cost8 = int(line[1]), int(line[2]), int(line[3]), float(line[4]), float(line[5])
    assert errors == 0 and nodes2 == 2 * n - 1 and total_ms > 0 and cost8 > 0
    assert "BVH2 build time" in run.stdout  # printed by BenchmarkBuild

    b2_cpp = np.fromfile(str(out) + ".bvh2", dtype=nxb.BVH2_NODE_DTYPE)
    b8_cpp = np.fromfile(str(out) + ".bvh8", dtype=nxb.BVH8_NODE_DTYPE)
    p_cpp = np.fromfile(str(out) + ".prim", dtype=np.uint32)
    assert b8_cpp.shape[0] == nodes8

    d = S.dev(prims.astype(np.float32))
    p2 = nxb.build_bvh2(d, nxb.BuildConfig())
    assert orc.compare_bvh2(b2_cpp, 2 * n - 2, S.nodes2(p2.nodes.view(-1)), 2 * n - 2, n) == 0
    p8 = nxb.build_bvh8(d, nxb.BuildConfig())
    b8_py = S.host(p8.nodes.reshape(-1)).view(nxb.BVH8_NODE_DTYPE)
    assert orc.compare_bvh8(b8_cpp, p_cpp, b8_py, S.host(p8.prim_idx).view(np.uint32), n) == 0
