"""GB300 (sm_103a) BVH builder: Python host side over the C ABI.

The build runs entirely in ``libnxb_gb300.so`` (hand-written CUDA kernels);
this module only binds its C ABI (``include/nxb_gb300.h``) with ctypes and
mirrors the reference's host interface (NexusBVH/include/NXB/BVHBuilder.h):

    build_bvh2(prims, config, metrics)  ~ NXB::BuildBVH2<PrimT>
    build_bvh8(prims, config, metrics)  ~ NXB::BuildBVH8<PrimT>

``prims`` is a CUDA tensor of float32 triangles ``[n, 9]`` (``NXB::Triangle``)
or boxes ``[n, 6]`` (``NXB::AABB``).  The returned BVHs hold CUDA tensors
whose bytes are the reference's node layouts.  There is no CPU path: if the
library is missing, importing the functions raises.
"""
from __future__ import annotations

import ctypes
import dataclasses
from pathlib import Path

import numpy as np

_LIB_PATH = Path(__file__).resolve().parent / "libnxb_gb300.so"
_lib = None

NXB_OK = 0
NXB_PRIM_AABB = 0
NXB_PRIM_TRIANGLE = 1
INVALID_IDX = 0xFFFFFFFF

STATUS_NAMES = {
    0: "NXB_OK", 1: "NXB_ERR_INVALID_ARGUMENT", 2: "NXB_ERR_UNSUPPORTED", 3: "NXB_ERR_OUT_OF_MEMORY",
    4: "NXB_ERR_CUDA", 5: "NXB_ERR_WORKSPACE_TOO_SMALL", 6: "NXB_ERR_DEVICE_TIMEOUT",
    7: "NXB_ERR_DEVICE_INVARIANT", 8: "NXB_ERR_ADMISSION", 9: "NXB_ERR_IO",
}

# numpy views of the device layouts
BVH2_NODE_DTYPE = np.dtype([("bmin", "<f4", 3), ("bmax", "<f4", 3), ("left", "<u4"), ("right", "<u4")])
BVH8_NODE_DTYPE = np.dtype([("p", "<f4", 3), ("e", "u1", 3), ("imask", "u1"), ("child_base", "<u4"),
                            ("prim_base", "<u4"), ("meta", "u1", 8), ("qlo", "u1", (3, 8)), ("qhi", "u1", (3, 8))])
assert BVH2_NODE_DTYPE.itemsize == 32 and BVH8_NODE_DTYPE.itemsize == 80


class NxbError(RuntimeError):
    def __init__(self, status: int, what: str = ""):
        self.status = status
        super().__init__(f"{what}: {STATUS_NAMES.get(status, status)}")


class CAABB(ctypes.Structure):
    _fields_ = [("bmin", ctypes.c_float * 3), ("bmax", ctypes.c_float * 3)]


class CBVH2(ctypes.Structure):
    _fields_ = [("nodes", ctypes.c_void_p), ("node_count", ctypes.c_uint32), ("prim_count", ctypes.c_uint32),
                ("bounds", CAABB)]


class CBVH8(ctypes.Structure):
    _fields_ = [("nodes", ctypes.c_void_p), ("node_count", ctypes.c_uint32), ("prim_idx", ctypes.c_void_p),
                ("prim_count", ctypes.c_uint32), ("bounds", CAABB)]


class CMetrics(ctypes.Structure):
    _fields_ = [(name, ctypes.c_float) for name in (
        "scene_bounds_time", "morton_codes_time", "radix_sort_time", "bvh2_build_time", "bvh8_conversion_time",
        "total_time", "bvh2_cost", "bvh8_cost", "average_child_per_node")]


class CConfig(ctypes.Structure):
    _fields_ = [("prioritize_speed", ctypes.c_uint32), ("search_radius", ctypes.c_uint32),
                ("flags", ctypes.c_uint32), ("reserved", ctypes.c_uint32)]


class CSizes(ctypes.Structure):
    _fields_ = [("workspace_bytes", ctypes.c_size_t), ("bvh2_node_count", ctypes.c_size_t),
                ("bvh8_node_capacity", ctypes.c_size_t)]


class CResult(ctypes.Structure):
    _fields_ = [("scene_bounds", CAABB), ("bvh8_node_count", ctypes.c_uint32), ("bvh8_leaf_count", ctypes.c_uint32),
                ("error_word", ctypes.c_uint32), ("bvh2_root", ctypes.c_uint32)]


class CBatchMesh(ctypes.Structure):
    _fields_ = [("scene_bounds", CAABB), ("prim_offset", ctypes.c_uint32), ("prim_count", ctypes.c_uint32),
                ("bvh2_offset", ctypes.c_uint32), ("bvh2_node_count", ctypes.c_uint32),
                ("bvh8_offset", ctypes.c_uint32), ("bvh8_node_count", ctypes.c_uint32),
                ("bvh8_leaf_count", ctypes.c_uint32)]


class CBatchArrays(ctypes.Structure):
    _fields_ = [("bvh2_nodes", ctypes.c_void_p), ("bvh8_nodes", ctypes.c_void_p), ("prim_idx", ctypes.c_void_p),
                ("meshes", ctypes.c_void_p), ("mesh_count", ctypes.c_uint32), ("prim_count", ctypes.c_uint32),
                ("bvh2_node_capacity", ctypes.c_size_t), ("bvh8_node_capacity", ctypes.c_size_t)]


class CBatchTuning(ctypes.Structure):
    _fields_ = [("sort_digit_bits", ctypes.c_uint32), ("search_radius", ctypes.c_uint32),
                ("hploc_ctas_per_sm", ctypes.c_uint32), ("fusion_groups", ctypes.c_uint32),
                ("block_size", ctypes.c_uint32), ("candidates_tried", ctypes.c_uint32),
                ("build_ms", ctypes.c_float)]


class CServerConfig(ctypes.Structure):
    _fields_ = [("memory_budget_bytes", ctypes.c_size_t), ("streams", ctypes.c_uint32),
                ("batch_max_prims", ctypes.c_uint32), ("batch_max_meshes", ctypes.c_uint32),
                ("flags", ctypes.c_uint32)]


class CServerResult(ctypes.Structure):
    _fields_ = [("bvh8", CBVH8), ("status", ctypes.c_int32), ("batched_with", ctypes.c_uint32),
                ("queue_ms", ctypes.c_double), ("latency_ms", ctypes.c_double),
                ("device_start_ms", ctypes.c_double), ("device_end_ms", ctypes.c_double)]


class CServerStats(ctypes.Structure):
    _fields_ = [(f, ctypes.c_uint64) for f in ("submitted", "completed", "rejected", "builds", "batched_builds",
                                               "batched_requests")] + \
               [("bytes_in_use", ctypes.c_size_t), ("peak_bytes_in_use", ctypes.c_size_t)]


assert ctypes.sizeof(CBVH2) == 40 and ctypes.sizeof(CBVH8) == 56 and ctypes.sizeof(CMetrics) == 36
assert ctypes.sizeof(CBatchMesh) == 52
NXB_TUNE_RADIUS = 0x1
NXB_BUILD_AUCTION = 0x1
NXB_BUILD_VALIDATE = 0x2
NXB_SERVER_RESERVE = 0x1

_P = ctypes.c_void_p
_U32 = ctypes.c_uint32
_SIG = {
    "nxb_status_string": (ctypes.c_char_p, [ctypes.c_int]),
    "nxb_last_cuda_error": (ctypes.c_int, []),
    "nxb_version": (ctypes.c_char_p, []),
    "nxb_build_bvh2": (ctypes.c_int, [_P, ctypes.c_int, _U32, _P, _P, ctypes.POINTER(CBVH2), _P]),
    "nxb_build_bvh8": (ctypes.c_int, [_P, ctypes.c_int, _U32, _P, _P, ctypes.POINTER(CBVH8), _P]),
    "nxb_bvh2_to_host": (ctypes.c_int, [ctypes.POINTER(CBVH2), ctypes.POINTER(CBVH2)]),
    "nxb_bvh8_to_host": (ctypes.c_int, [ctypes.POINTER(CBVH8), ctypes.POINTER(CBVH8)]),
    "nxb_free_host_bvh2": (ctypes.c_int, [ctypes.POINTER(CBVH2)]),
    "nxb_free_host_bvh8": (ctypes.c_int, [ctypes.POINTER(CBVH8)]),
    "nxb_write_bvh2": (ctypes.c_int, [ctypes.c_char_p, ctypes.POINTER(CBVH2)]),
    "nxb_read_bvh2": (ctypes.c_int, [ctypes.c_char_p, ctypes.POINTER(CBVH2)]),
    "nxb_write_bvh8": (ctypes.c_int, [ctypes.c_char_p, ctypes.POINTER(CBVH8)]),
    "nxb_read_bvh8": (ctypes.c_int, [ctypes.c_char_p, ctypes.POINTER(CBVH8)]),
    "nxb_free_device_bvh2": (ctypes.c_int, [ctypes.POINTER(CBVH2)]),
    "nxb_free_device_bvh8": (ctypes.c_int, [ctypes.POINTER(CBVH8)]),
    "nxb_query_build_sizes": (ctypes.c_int, [_U32, _P, ctypes.POINTER(CSizes)]),
    "nxb_build_async": (ctypes.c_int, [_P, ctypes.c_int, _U32, _P, _P, ctypes.c_size_t, _P, _P, _P, _P, _P]),
    "nxb_build_async_timed": (ctypes.c_int, [_P, ctypes.c_int, _U32, _P, _P, ctypes.c_size_t, _P, _P, _P, _P, _P,
                                             _P]),
    "nxb_stage_scene_bounds": (ctypes.c_int, [_P, ctypes.c_int, _U32, _P, _P, _P]),
    "nxb_stage_morton": (ctypes.c_int, [_P, _U32, _P, _U32, _P, _P, _P]),
    "nxb_sort_scratch_bytes": (ctypes.c_size_t, [_U32, _U32, _U32, _U32]),
    "nxb_stage_radix_sort": (ctypes.c_int, [_U32, _P, _P, _P, _P, _U32, _U32, _U32, _P, ctypes.c_size_t, _P, _P]),
    "nxb_hploc_scratch_bytes": (ctypes.c_size_t, [_U32]),
    "nxb_stage_hploc": (ctypes.c_int, [_U32, _P, _P, _P, _U32, _U32, _P, ctypes.c_size_t, _P, _P]),
    "nxb_bvh8_scratch_bytes": (ctypes.c_size_t, [_U32]),
    "nxb_stage_bvh8": (ctypes.c_int, [_P, _U32, _P, _P, _P, _P, ctypes.c_size_t, _P, _P]),
    "nxb_stage_bvh8_ex": (ctypes.c_int, [_P, _U32, _P, _P, _P, _P, ctypes.c_size_t, _U32, _P, _P]),
    "nxb_eval_bvh2_cost": (ctypes.c_int, [_P, _U32, _P, _P, _P]),
    "nxb_eval_bvh8_cost": (ctypes.c_int, [_P, _U32, _P, _P, _P]),
    "nxb_validate_bvh2_scratch_bytes": (ctypes.c_size_t, [_U32]),
    "nxb_validate_bvh2": (ctypes.c_int, [_P, _U32, _U32, _P, _P, ctypes.c_size_t, _P]),
    "nxb_validate_bvh8_scratch_bytes": (ctypes.c_size_t, [_U32, _U32]),
    "nxb_validate_bvh8": (ctypes.c_int, [_P, _U32, _P, _U32, _P, ctypes.c_int, _P, _P, ctypes.c_size_t, _P]),
    "nxb_selftest_numerics": (ctypes.c_int, [_P, _U32]),
    "nxb_selftest_bounded_waits": (ctypes.c_int, [_P]),
    "nxb_batch_create": (ctypes.c_int, [ctypes.c_int, _P, _U32, _P, ctypes.POINTER(ctypes.c_void_p)]),
    "nxb_batch_destroy": (ctypes.c_int, [_P]),
    "nxb_batch_build_async": (ctypes.c_int, [_P, _P, _P]),
    "nxb_batch_wait": (ctypes.c_int, [_P, _P, _P]),
    "nxb_batch_build": (ctypes.c_int, [_P, _P, _P, _P]),
    "nxb_batch_get_arrays": (ctypes.c_int, [_P, ctypes.POINTER(CBatchArrays)]),
    "nxb_batch_autotune": (ctypes.c_int, [_P, _P, _U32, _U32, _P, ctypes.POINTER(CBatchTuning)]),
    "nxb_batch_set_tuning": (ctypes.c_int, [_P, ctypes.POINTER(CBatchTuning)]),
    "nxb_batch_get_tuning": (ctypes.c_int, [_P, ctypes.POINTER(CBatchTuning)]),
    "nxb_batch_mesh_bvh8_to_host": (ctypes.c_int, [_P, _U32, ctypes.POINTER(CBVH8)]),
    "nxb_server_create": (ctypes.c_int, [ctypes.POINTER(CServerConfig), ctypes.POINTER(ctypes.c_void_p)]),
    "nxb_server_destroy": (ctypes.c_int, [_P]),
    "nxb_server_submit": (ctypes.c_int, [_P, _P, ctypes.c_int, ctypes.c_int, _U32, _P,
                                         ctypes.POINTER(ctypes.c_uint64)]),
    "nxb_server_wait": (ctypes.c_int, [_P, ctypes.c_uint64, ctypes.POINTER(CServerResult)]),
    "nxb_server_poll": (ctypes.c_int, [_P, ctypes.c_uint64, ctypes.POINTER(CServerResult),
                                       ctypes.POINTER(ctypes.c_int)]),
    "nxb_server_release": (ctypes.c_int, [_P, ctypes.c_uint64]),
    "nxb_server_get_stats": (ctypes.c_int, [_P, ctypes.POINTER(CServerStats)]),
}


def lib_path() -> Path:
    return _LIB_PATH


def load() -> ctypes.CDLL:
    """Loads libnxb_gb300.so (built by ``__graft_entry__.build()``); raises if absent."""
    global _lib
    if _lib is None:
        if not _LIB_PATH.exists():
            raise RuntimeError(f"{_LIB_PATH.name} is not built: run __graft_entry__.build() (there is no CPU path)")
        lib = ctypes.CDLL(str(_LIB_PATH))
        for name, (res, args) in _SIG.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
    return _lib


def check(status: int, what: str) -> None:
    if status != NXB_OK:
        raise NxbError(status, what)


def _stream_ptr(stream=None) -> int:
    import torch
    s = stream if stream is not None else torch.cuda.current_stream()
    return int(s.cuda_stream)


@dataclasses.dataclass
class BuildConfig:
    """NXB::BuildConfig plus the H-PLOC search radius and the BVH8 auction
    assignment (both compile-time in the reference)."""
    prioritize_speed: bool = False
    search_radius: int = 8
    auction: bool = False
    validate: bool = False  # plain builds: check the trees on the device before returning

    def to_c(self) -> CConfig:
        flags = (NXB_BUILD_AUCTION if self.auction else 0) | (NXB_BUILD_VALIDATE if self.validate else 0)
        return CConfig(1 if self.prioritize_speed else 0, int(self.search_radius), flags, 0)

    @property
    def key_bits(self) -> int:
        return 30 if self.prioritize_speed else 63


@dataclasses.dataclass
class BVHBuildMetrics:
    """NXB::BVHBuildMetrics: per-stage CUDA-event milliseconds and costs."""
    scene_bounds_time: float = 0.0
    morton_codes_time: float = 0.0
    radix_sort_time: float = 0.0
    bvh2_build_time: float = 0.0
    bvh8_conversion_time: float = 0.0
    total_time: float = 0.0
    bvh2_cost: float = 0.0
    bvh8_cost: float = 0.0
    average_child_per_node: float = 0.0

    @classmethod
    def from_c(cls, m: CMetrics) -> "BVHBuildMetrics":
        return cls(**{f.name: float(getattr(m, f.name)) for f in dataclasses.fields(cls)})


def prim_type_of(prims) -> int:
    if prims.dim() != 2 or prims.shape[1] not in (6, 9):
        raise ValueError("prims must be [n, 9] float32 triangles or [n, 6] float32 boxes")
    return NXB_PRIM_TRIANGLE if prims.shape[1] == 9 else NXB_PRIM_AABB


@dataclasses.dataclass
class BVH2:
    nodes: object          # torch uint8 CUDA tensor [2n-1, 32]
    node_count: int
    prim_count: int
    bounds: tuple          # (bmin, bmax)

    @property
    def root(self) -> int:
        return self.node_count - 1


@dataclasses.dataclass
class BVH8:
    nodes: object          # torch uint8 CUDA tensor [node_count, 80]
    node_count: int
    prim_idx: object       # torch int32 CUDA tensor [n]
    prim_count: int
    bounds: tuple
    bvh2: BVH2 | None = None


class Builder:
    """Keeps a workspace resident across builds and drives ``nxb_build_async``.

    The build enqueues on the current torch stream with no allocation inside
    the library; results are torch CUDA tensors.
    """

    def __init__(self):
        load()
        self._ws = None

    def sizes(self, n: int, config: BuildConfig) -> CSizes:
        s = CSizes()
        c = config.to_c()
        check(load().nxb_query_build_sizes(n, ctypes.byref(c), ctypes.byref(s)), "nxb_query_build_sizes")
        return s

    def workspace(self, nbytes: int):
        import torch
        if self._ws is None or self._ws.numel() < nbytes:
            self._ws = torch.empty(nbytes, dtype=torch.uint8, device="cuda")
        return self._ws

    def enqueue(self, prims, n, config, ws, bvh2_nodes, bvh8_nodes, prim_idx, result, stream=None) -> None:
        c = config.to_c()
        check(load().nxb_build_async(
            prims.data_ptr(), prim_type_of(prims), n, ctypes.byref(c), ws.data_ptr(), ws.numel(),
            bvh2_nodes.data_ptr(), bvh8_nodes.data_ptr() if bvh8_nodes is not None else None,
            prim_idx.data_ptr() if prim_idx is not None else None, result.data_ptr(), _stream_ptr(stream)),
            "nxb_build_async")

    def build(self, prims, config: BuildConfig = BuildConfig(), wide: bool = True):
        import torch
        n = int(prims.shape[0])
        s = self.sizes(n, config)
        ws = self.workspace(s.workspace_bytes)
        bvh2_nodes = torch.empty((s.bvh2_node_count, 32), dtype=torch.uint8, device="cuda")
        bvh8_nodes = torch.empty((s.bvh8_node_capacity, 80), dtype=torch.uint8, device="cuda") if wide else None
        prim_idx = torch.empty(n, dtype=torch.int32, device="cuda") if wide else None
        result = torch.zeros(ctypes.sizeof(CResult), dtype=torch.uint8, device="cuda")
        self.enqueue(prims, n, config, ws, bvh2_nodes, bvh8_nodes, prim_idx, result)
        r = CResult.from_buffer_copy(result.cpu().numpy().tobytes())
        if r.error_word:
            raise NxbError(7 if not (r.error_word & 3) else 6, f"device error word 0x{r.error_word:x}")
        bounds = (tuple(r.scene_bounds.bmin), tuple(r.scene_bounds.bmax))
        b2 = BVH2(bvh2_nodes, int(s.bvh2_node_count), n, bounds)
        if not wide:
            return b2
        return BVH8(bvh8_nodes[: r.bvh8_node_count], int(r.bvh8_node_count), prim_idx, n, bounds, b2)


def build_bvh2(prims, config: BuildConfig = BuildConfig(), metrics: BVHBuildMetrics | None = None) -> BVH2:
    """NXB::BuildBVH2 through ``nxb_build_bvh2`` (library-owned output, copied into a torch tensor)."""
    out = _build_plain(prims, config, metrics, wide=False)
    return out


def build_bvh8(prims, config: BuildConfig = BuildConfig(), metrics: BVHBuildMetrics | None = None) -> BVH8:
    """NXB::BuildBVH8 through ``nxb_build_bvh8`` (library-owned output, copied into torch tensors)."""
    return _build_plain(prims, config, metrics, wide=True)


def _build_plain(prims, config, metrics, wide):
    import torch
    lib = load()
    n = int(prims.shape[0])
    c = config.to_c()
    m = CMetrics()
    mp = ctypes.byref(m) if metrics is not None else None
    stream = _stream_ptr()
    if wide:
        out = CBVH8()
        check(lib.nxb_build_bvh8(prims.data_ptr(), prim_type_of(prims), n, ctypes.byref(c), stream,
                                 ctypes.byref(out), mp), "nxb_build_bvh8")
        nodes = torch.empty((out.node_count, 80), dtype=torch.uint8, device="cuda")
        prim_idx = torch.empty(n, dtype=torch.int32, device="cuda")
        _copy_d2d(nodes.data_ptr(), out.nodes, out.node_count * 80)
        _copy_d2d(prim_idx.data_ptr(), out.prim_idx, n * 4)
        bounds = (tuple(out.bounds.bmin), tuple(out.bounds.bmax))
        check(lib.nxb_free_device_bvh8(ctypes.byref(out)), "nxb_free_device_bvh8")
        res = BVH8(nodes, int(out.node_count), prim_idx, n, bounds)
    else:
        out = CBVH2()
        check(lib.nxb_build_bvh2(prims.data_ptr(), prim_type_of(prims), n, ctypes.byref(c), stream,
                                 ctypes.byref(out), mp), "nxb_build_bvh2")
        nodes = torch.empty((out.node_count, 32), dtype=torch.uint8, device="cuda")
        _copy_d2d(nodes.data_ptr(), out.nodes, out.node_count * 32)
        bounds = (tuple(out.bounds.bmin), tuple(out.bounds.bmax))
        check(lib.nxb_free_device_bvh2(ctypes.byref(out)), "nxb_free_device_bvh2")
        res = BVH2(nodes, int(out.node_count), n, bounds)
    if metrics is not None:
        for f in dataclasses.fields(BVHBuildMetrics):
            setattr(metrics, f.name, float(getattr(m, f.name)))
    return res


def _copy_d2d(dst: int, src: int, nbytes: int) -> None:
    import torch
    if nbytes == 0:
        return
    # wrap the library-owned pointer without taking ownership
    src_t = _borrow(src, nbytes)
    dst_t = _borrow(dst, nbytes)
    dst_t.copy_(src_t)
    torch.cuda.synchronize()


def _borrow(ptr: int, nbytes: int):
    import torch
    cls = type("_CudaArray", (), {})
    obj = cls()
    obj.__cuda_array_interface__ = {"shape": (nbytes,), "typestr": "|u1", "data": (ptr, False), "version": 3,
                                    "strides": None}
    return torch.as_tensor(obj, device="cuda")


class Batch:
    """Batched builds of many independent meshes (``nxb_batch_*``).

    ``counts`` are the meshes' primitive counts; ``build(prims)`` takes all
    meshes' primitives end to end in one CUDA tensor and builds every mesh
    exactly as ``build_bvh8`` would build it alone (30-bit codes only).
    """

    def __init__(self, counts, prim_type: int = NXB_PRIM_TRIANGLE, config: BuildConfig | None = None):
        lib = load()
        config = config or BuildConfig(prioritize_speed=True)
        counts = np.asarray(counts, dtype=np.uint64)
        off = np.zeros(len(counts) + 1, dtype=np.uint32)
        off[1:] = np.cumsum(counts).astype(np.uint32)
        self.offsets = off
        self.mesh_count = len(counts)
        self._handle = ctypes.c_void_p()
        c = config.to_c()
        check(lib.nxb_batch_create(prim_type, off.ctypes.data, self.mesh_count, ctypes.byref(c),
                                   ctypes.byref(self._handle)), "nxb_batch_create")

    def close(self) -> None:
        if self._handle:
            load().nxb_batch_destroy(self._handle)
            self._handle = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def build_async(self, prims, stream=None) -> None:
        check(load().nxb_batch_build_async(self._handle, prims.data_ptr(), _stream_ptr(stream)),
              "nxb_batch_build_async")

    def wait(self, stream=None, results: bool = True):
        meshes = (CBatchMesh * self.mesh_count)() if results else None
        check(load().nxb_batch_wait(self._handle, _stream_ptr(stream),
                                    ctypes.cast(meshes, ctypes.c_void_p) if results else None), "nxb_batch_wait")
        return list(meshes) if results else None

    def build(self, prims, stream=None):
        self.build_async(prims, stream)
        return self.wait(stream)

    def autotune(self, prims, flags: int = 0, repeats: int = 3, stream=None) -> CBatchTuning:
        t = CBatchTuning()
        check(load().nxb_batch_autotune(self._handle, prims.data_ptr(), flags, repeats, _stream_ptr(stream),
                                        ctypes.byref(t)), "nxb_batch_autotune")
        return t

    def tuning(self) -> CBatchTuning:
        t = CBatchTuning()
        check(load().nxb_batch_get_tuning(self._handle, ctypes.byref(t)), "nxb_batch_get_tuning")
        return t

    def set_tuning(self, t: CBatchTuning) -> None:
        check(load().nxb_batch_set_tuning(self._handle, ctypes.byref(t)), "nxb_batch_set_tuning")

    def arrays(self) -> CBatchArrays:
        a = CBatchArrays()
        check(load().nxb_batch_get_arrays(self._handle, ctypes.byref(a)), "nxb_batch_get_arrays")
        return a

    def mesh_bvh8_host(self, mesh: int):
        """(nodes as BVH8_NODE_DTYPE array, prim_idx uint32 array) of one mesh."""
        lib = load()
        h = CBVH8()
        check(lib.nxb_batch_mesh_bvh8_to_host(self._handle, mesh, ctypes.byref(h)), "nxb_batch_mesh_bvh8_to_host")
        try:
            nodes = np.frombuffer(ctypes.string_at(h.nodes, h.node_count * 80), dtype=BVH8_NODE_DTYPE).copy()
            prim = np.frombuffer(ctypes.string_at(h.prim_idx, h.prim_count * 4), dtype=np.uint32).copy()
        finally:
            lib.nxb_free_host_bvh8(ctypes.byref(h))
        return nodes, prim

    def validate_mesh(self, mesh: int, prims, meshes=None):
        """Checks one mesh's BVH2 and BVH8 on the device, in place in the
        batch's arrays (their indices are mesh-local, so each mesh is a
        standalone tree); ``prims`` is the CUDA tensor the batch was built
        from.  Returns ((errors, report) of the BVH2, (errors, report) of the
        BVH8)."""
        a = self.arrays()
        info = (meshes or self.wait(results=True))[mesh]
        n = int(info.prim_count)
        if n == 0:
            raise ValueError("an empty mesh has no tree")
        b2 = _borrow(a.bvh2_nodes + info.bvh2_offset * 32, info.bvh2_node_count * 32)
        b8 = _borrow(a.bvh8_nodes + info.bvh8_offset * 80, info.bvh8_node_count * 80)
        pi = _borrow(a.prim_idx + info.prim_offset * 4, n * 4)
        pm = prims[info.prim_offset:info.prim_offset + n]
        return validate_bvh2(b2, n), validate_bvh8(b8, int(info.bvh8_node_count), pi, pm)

    def mesh_bvh2_host(self, mesh: int, meshes=None):
        """BVH2 nodes (BVH2_NODE_DTYPE, mesh-local child indices) of one mesh after a build."""
        import torch
        a = self.arrays()
        info = (meshes or self.wait(results=True))[mesh]
        nbytes = info.bvh2_node_count * 32
        if nbytes == 0:
            return np.zeros(0, dtype=BVH2_NODE_DTYPE)
        t = _borrow(a.bvh2_nodes + info.bvh2_offset * 32, nbytes)
        torch.cuda.synchronize()
        return np.frombuffer(t.cpu().numpy().tobytes(), dtype=BVH2_NODE_DTYPE).copy()


class Server:
    """Build server (``nxb_server_*``): continuous batching under a memory budget.

    ``submit`` takes a numpy array (host input, kept alive here until the
    request completes) or a CUDA tensor (device input) and returns a ticket;
    ``wait`` returns the ``CServerResult`` whose ``bvh8`` points into server
    memory until ``release``.
    """

    def __init__(self, budget_bytes: int = 0, streams: int = 0, batch_max_prims: int = 0, batch_max_meshes: int = 0,
                 reserve: bool = False):
        self._h = ctypes.c_void_p()
        c = CServerConfig(budget_bytes, streams, batch_max_prims, batch_max_meshes, NXB_SERVER_RESERVE if reserve else 0)
        check(load().nxb_server_create(ctypes.byref(c), ctypes.byref(self._h)), "nxb_server_create")
        self._keep = {}

    def close(self) -> None:
        if self._h:
            load().nxb_server_destroy(self._h)
            self._h = ctypes.c_void_p()
            self._keep.clear()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def submit(self, prims, config: BuildConfig = BuildConfig()) -> int:
        t = ctypes.c_uint64()
        c = config.to_c()
        if isinstance(prims, np.ndarray):
            prims = np.ascontiguousarray(prims, dtype=np.float32)
            ptr, on_dev, n, kind = prims.ctypes.data, 0, prims.shape[0], prims.shape[1]
        else:
            ptr, on_dev, n, kind = prims.data_ptr(), 1, int(prims.shape[0]), int(prims.shape[1])
        ptype = NXB_PRIM_TRIANGLE if kind == 9 else NXB_PRIM_AABB
        check(load().nxb_server_submit(self._h, ptr, on_dev, ptype, n, ctypes.byref(c), ctypes.byref(t)),
              "nxb_server_submit")
        self._keep[t.value] = prims
        return t.value

    def wait(self, ticket: int) -> CServerResult:
        r = CServerResult()
        st = load().nxb_server_wait(self._h, ticket, ctypes.byref(r))
        self._keep.pop(ticket, None)
        check(st, "nxb_server_wait")
        return r

    def poll(self, ticket: int):
        r = CServerResult()
        done = ctypes.c_int()
        check(load().nxb_server_poll(self._h, ticket, ctypes.byref(r), ctypes.byref(done)), "nxb_server_poll")
        return r if done.value else None

    def release(self, ticket: int) -> None:
        check(load().nxb_server_release(self._h, ticket), "nxb_server_release")

    def stats(self) -> CServerStats:
        s = CServerStats()
        check(load().nxb_server_get_stats(self._h, ctypes.byref(s)), "nxb_server_get_stats")
        return s

    @staticmethod
    def bvh8_host(result: CServerResult):
        """(nodes, prim_idx) numpy copies of a result's BVH8."""
        lib = load()
        h = CBVH8()
        b = result.bvh8
        check(lib.nxb_bvh8_to_host(ctypes.byref(b), ctypes.byref(h)), "nxb_bvh8_to_host")
        try:
            nodes = np.frombuffer(ctypes.string_at(h.nodes, h.node_count * 80), dtype=BVH8_NODE_DTYPE).copy()
            prim = np.frombuffer(ctypes.string_at(h.prim_idx, h.prim_count * 4), dtype=np.uint32).copy()
        finally:
            lib.nxb_free_host_bvh8(ctypes.byref(h))
        return nodes, prim


def _caabb(bounds) -> CAABB:
    b = np.asarray(bounds, dtype=np.float32).reshape(2, 3)
    return CAABB((ctypes.c_float * 3)(*b[0]), (ctypes.c_float * 3)(*b[1]))


def save_bvh2(path, nodes: np.ndarray, bounds) -> None:
    """Writes host BVH2 nodes (BVH2_NODE_DTYPE, 2n-1 of them) and the root
    bounds ((2, 3): min, max) to a BVH file (nxb_write_bvh2)."""
    nodes = np.ascontiguousarray(nodes, dtype=BVH2_NODE_DTYPE)
    h = CBVH2(nodes.ctypes.data, len(nodes), (len(nodes) + 1) // 2, _caabb(bounds))
    check(load().nxb_write_bvh2(str(path).encode(), ctypes.byref(h)), "nxb_write_bvh2")


def load_bvh2(path):
    """(nodes as BVH2_NODE_DTYPE array, bounds (2, 3)) read from a BVH file."""
    lib = load()
    h = CBVH2()
    check(lib.nxb_read_bvh2(str(path).encode(), ctypes.byref(h)), "nxb_read_bvh2")
    try:
        nodes = np.frombuffer(ctypes.string_at(h.nodes, h.node_count * 32), dtype=BVH2_NODE_DTYPE).copy()
    finally:
        lib.nxb_free_host_bvh2(ctypes.byref(h))
    return nodes, np.array([list(h.bounds.bmin), list(h.bounds.bmax)], dtype=np.float32)


def save_bvh8(path, nodes: np.ndarray, prim_idx: np.ndarray, bounds) -> None:
    """Writes host BVH8 nodes (BVH8_NODE_DTYPE), prim_idx and the root bounds
    to a BVH file (nxb_write_bvh8)."""
    nodes = np.ascontiguousarray(nodes, dtype=BVH8_NODE_DTYPE)
    prim = np.ascontiguousarray(prim_idx, dtype=np.uint32)
    h = CBVH8(nodes.ctypes.data, len(nodes), prim.ctypes.data, len(prim), _caabb(bounds))
    check(load().nxb_write_bvh8(str(path).encode(), ctypes.byref(h)), "nxb_write_bvh8")


def load_bvh8(path):
    """(nodes as BVH8_NODE_DTYPE array, prim_idx uint32 array, bounds (2, 3))
    read from a BVH file."""
    lib = load()
    h = CBVH8()
    check(lib.nxb_read_bvh8(str(path).encode(), ctypes.byref(h)), "nxb_read_bvh8")
    try:
        nodes = np.frombuffer(ctypes.string_at(h.nodes, h.node_count * 80), dtype=BVH8_NODE_DTYPE).copy()
        prim = np.frombuffer(ctypes.string_at(h.prim_idx, h.prim_count * 4), dtype=np.uint32).copy()
    finally:
        lib.nxb_free_host_bvh8(ctypes.byref(h))
    return nodes, prim, np.array([list(h.bounds.bmin), list(h.bounds.bmax)], dtype=np.float32)


BVH2_CHECK_FIELDS = ("reached", "leaves", "dup_prims", "missing_prims", "bad_union", "not_contained", "bad_index",
                     "max_depth", "extra_parents", "errors")
BVH8_CHECK_FIELDS = ("reached", "leaves", "dup_prims", "missing_prims", "bad_index", "lo_not_conservative",
                     "hi_not_conservative", "slots_used", "max_depth", "meta_errors", "errors")


def _device_bytes(t, what: str) -> int:
    """Bytes a CUDA tensor holds; raises unless it is contiguous on a CUDA device."""
    if not t.is_cuda or not t.is_contiguous():
        raise ValueError(f"{what} must be a contiguous CUDA tensor")
    return t.numel() * t.element_size()


def _run_check(fn, fields, scratch_bytes, args, device, stream):
    import torch
    if scratch_bytes == 0:
        raise ValueError("sizes out of range for the validator")
    s = stream if stream is not None else torch.cuda.current_stream(device)
    with torch.cuda.stream(s):
        scratch = torch.empty(scratch_bytes, dtype=torch.uint8, device=device)
        report = torch.empty(len(fields), dtype=torch.int64, device=device)
        check(fn(*args, report.data_ptr(), scratch.data_ptr(), scratch_bytes, int(s.cuda_stream)), fn.__name__)
        s.synchronize()
    rep = dict(zip(fields, (int(v) for v in report.cpu().numpy().view(np.uint64))))
    return rep["errors"], rep


def validate_bvh2(nodes, prim_count: int, root: int | None = None, stream=None):
    """Checks a BVH2 on the device (nxb_validate_bvh2): ``nodes`` is a CUDA
    tensor holding the 2n-1 nodes (32 bytes each), ``root`` defaults to 2n-2.
    Returns (errors, report); the tree is valid when errors is 0."""
    lib = load()
    n = int(prim_count)
    root = 2 * n - 2 if root is None else int(root)
    if _device_bytes(nodes, "nodes") < (2 * n - 1) * 32:
        raise ValueError("nodes holds fewer than 2n-1 BVH2 nodes")
    return _run_check(lib.nxb_validate_bvh2, BVH2_CHECK_FIELDS, lib.nxb_validate_bvh2_scratch_bytes(n),
                      (nodes.data_ptr(), n, root), nodes.device, stream)


def validate_bvh8(nodes, node_count: int, prim_idx, prims, stream=None):
    """Checks a BVH8 on the device (nxb_validate_bvh8): ``nodes`` (80-byte
    nodes, root 0) and ``prim_idx`` are CUDA tensors, ``prims`` the CUDA
    tensor the tree was built over ([n, 9] triangles or [n, 6] boxes, whose
    boxes the quantised child bounds are checked against).  Returns (errors,
    report); the tree is valid when errors is 0."""
    import torch
    lib = load()
    n = int(prims.shape[0])
    m = int(node_count)
    if _device_bytes(nodes, "nodes") < m * 80:
        raise ValueError("nodes holds fewer than node_count BVH8 nodes")
    if _device_bytes(prim_idx, "prim_idx") < n * 4:
        raise ValueError("prim_idx holds fewer than n entries")
    if prims.dtype != torch.float32:
        raise ValueError("prims must be float32")
    _device_bytes(prims, "prims")
    return _run_check(lib.nxb_validate_bvh8, BVH8_CHECK_FIELDS, lib.nxb_validate_bvh8_scratch_bytes(m, n),
                      (nodes.data_ptr(), m, prim_idx.data_ptr(), n, prims.data_ptr(), prim_type_of(prims)),
                      nodes.device, stream)


def selftest_numerics() -> list[int]:
    rep = (ctypes.c_uint32 * 40)()
    check(load().nxb_selftest_numerics(ctypes.cast(rep, ctypes.c_void_p), 40), "nxb_selftest_numerics")
    return list(rep)


def version() -> str:
    return load().nxb_version().decode()
