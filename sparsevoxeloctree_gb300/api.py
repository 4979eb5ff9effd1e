"""Host-side mirror of the reference's hot-path classes over the C ABI.

Voxelizer, OctreeBuilder, Octree and OctreeTracer keep the reference's names and call shapes
(src/Voxelizer.hpp:43-52, src/OctreeBuilder.hpp:36-43, src/Octree.hpp:18-28, src/OctreeTracer.hpp:57-70);
`Cmd*` methods become stream-ordered calls and device memory is torch tensors (plumbing only: every
computation is a libsvo.so kernel).  Status codes other than SVO_OK raise SvoError.
"""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _lib
from .formats import CAMERA_DTYPE, HIT_DTYPE, RAY_DTYPE, TRIANGLE_DTYPE


def _stream(stream=None) -> ctypes.c_void_p:
    s = stream if stream is not None else torch.cuda.current_stream()
    return ctypes.c_void_p(s.cuda_stream)


def _ptr(t: torch.Tensor | None) -> ctypes.c_void_p:
    return ctypes.c_void_p(t.data_ptr() if t is not None else 0)


def to_device(arr: np.ndarray, device="cuda") -> torch.Tensor:
    """Upload a structured numpy array (triangles, rays, ...) as raw bytes."""
    a = np.ascontiguousarray(arr)
    return torch.from_numpy(a.view(np.uint8).reshape(-1)).to(device)


def from_device(t: torch.Tensor, dtype: np.dtype) -> np.ndarray:
    return t.detach().cpu().numpy().view(np.uint8).view(dtype)


def camera_struct(cam) -> _lib.CameraC:
    c = np.asarray(cam, CAMERA_DTYPE).reshape(())
    out = _lib.CameraC()
    for k in ("pos", "look", "side", "up"):
        getattr(out, k)[:] = [float(x) for x in c[k]]
    return out


class TorchAllocator:
    """Routes the engine's device allocations through torch's caching allocator (svo_allocator)."""

    def __init__(self, device):
        self.device = torch.device(device)
        self.live: dict[int, torch.Tensor] = {}
        self._alloc = _lib.ALLOC_FN(self._on_alloc)
        self._release = _lib.RELEASE_FN(self._on_release)
        self.struct = _lib.Allocator(self._alloc, self._release, None)

    def _on_alloc(self, user, nbytes):
        try:
            t = torch.empty(int(nbytes), dtype=torch.uint8, device=self.device)
        except RuntimeError:
            return None
        self.live[t.data_ptr()] = t
        return t.data_ptr()

    def _on_release(self, user, ptr):
        self.live.pop(ptr, None)

    def take(self, ptr: int) -> torch.Tensor:
        return self.live.pop(ptr)


# ------------------------------------------------------------------------------------------- Voxelizer
class Voxelizer:
    """Voxelizer (src/Voxelizer.hpp:13-53): triangles -> voxel-fragment list at a level."""

    def __init__(self):
        self.m_level = 0
        self.m_voxel_resolution = 0
        self.m_voxel_fragment_count = 0
        self.m_tris: torch.Tensor | None = None
        self.m_n_tris = 0
        self.m_voxel_fragment_list: torch.Tensor | None = None
        self.m_workspace: torch.Tensor | None = None
        self.m_count_dev: torch.Tensor | None = None
        self.m_units = 0

    @staticmethod
    def Create(triangles, octree_level: int, stream=None) -> "Voxelizer":
        """Voxelizer::Create (src/Voxelizer.cpp:5-26): count pass, exact allocation, then the fragment
        list is filled (the reference records that second pass in CmdVoxelize)."""
        v = Voxelizer()
        if isinstance(triangles, np.ndarray):
            triangles = to_device(np.asarray(triangles, TRIANGLE_DTYPE))
        v.m_tris = triangles
        v.m_n_tris = triangles.numel() // TRIANGLE_DTYPE.itemsize
        v.m_level = int(octree_level)
        v.m_voxel_resolution = 1 << v.m_level
        lib = _lib.load()
        alloc = TorchAllocator(triangles.device)
        out = _lib.Fraglist()
        _lib.check(lib.svo_voxelize_ex(_ptr(triangles), v.m_n_tris, v.m_level, ctypes.byref(alloc.struct),
                                       ctypes.byref(out), _stream(stream)))
        v.m_voxel_fragment_count = int(out.count)
        v.m_units = int(out.units)
        buf = alloc.take(out.data) if out.count else torch.empty(0, dtype=torch.uint8, device=triangles.device)
        v.m_voxel_fragment_list = buf.view(torch.int64)[: out.count]
        return v

    def CmdVoxelize(self, stream=None) -> None:
        """Voxelizer::CmdVoxelize (src/Voxelizer.cpp:167-179): emit the fragments again into the list."""
        lib = _lib.load()
        if self.m_workspace is None:
            dev = self.m_tris.device
            self.m_workspace = torch.empty(lib.svo_voxelize_workspace_size(self.m_n_tris, self.m_units),
                                           dtype=torch.uint8, device=dev)
            self.m_count_dev = torch.zeros(2, dtype=torch.int64, device=dev)
        _lib.check(lib.svo_voxelize_into(_ptr(self.m_tris), self.m_n_tris, self.m_level,
                                         _ptr(self.m_voxel_fragment_list), self.m_voxel_fragment_count,
                                         _ptr(self.m_count_dev), _ptr(self.m_workspace), self.m_workspace.numel(),
                                         _stream(stream)))

    def CheckEmission(self) -> None:
        """Raise unless the last CmdVoxelize produced every fragment (blocking read)."""
        count, status = (int(x) for x in self.m_count_dev.cpu())
        if status != 0 or count != self.m_voxel_fragment_count:
            raise _lib.SvoError(_lib.SVO_ERR_CAPACITY,
                                f"re-emission incomplete: {count} of {self.m_voxel_fragment_count} fragments, "
                                f"status {status}")

    def GetLevel(self) -> int:
        return self.m_level

    def GetVoxelResolution(self) -> int:
        return self.m_voxel_resolution

    def GetVoxelFragmentCount(self) -> int:
        return self.m_voxel_fragment_count

    def GetVoxelFragmentList(self) -> torch.Tensor:
        """Device tensor (int64 view of the uint64 fragments: low word x, high word y)."""
        return self.m_voxel_fragment_list


# ------------------------------------------------------------------------------------------- OctreeBuilder
class OctreeBuilder:
    """OctreeBuilder (src/OctreeBuilder.hpp:13-49): fragments -> node pool, level by level."""

    RESULT_WORDS = ctypes.sizeof(_lib.BuildInfo) // 4 + 1

    def __init__(self):
        self.m_voxelizer: Voxelizer | None = None
        self.m_fragments: torch.Tensor | None = None
        self.m_count = 0
        self.m_level = 0
        self.m_capacity = 0
        self.m_octree_buffer: torch.Tensor | None = None
        self.m_workspace: torch.Tensor | None = None
        self.m_result: torch.Tensor | None = None
        self._info: dict | None = None

    @staticmethod
    def Create(voxelizer: Voxelizer | None = None, fragments: torch.Tensor | None = None, level: int | None = None,
               capacity: int | None = None, leaf_words: int | None = None) -> "OctreeBuilder":
        """OctreeBuilder::Create (src/OctreeBuilder.cpp:8-50): allocates the node pool and scratch.  The pool
        holds the exact upper bound on the words a build of these fragments can use (the reference
        guesses F*floor(L/3) words and writes past the buffer when the guess is short); Reserve() shrinks
        it to the exact range after a first build.  `leaf_words` is accepted for compatibility: the leaf
        level needs no device scratch."""
        b = OctreeBuilder()
        if voxelizer is not None:
            b.m_voxelizer = voxelizer
            fragments = voxelizer.GetVoxelFragmentList()
            level = voxelizer.GetLevel()
        b.m_fragments = fragments
        b.m_count = int(fragments.numel())
        b.m_level = int(level)
        lib = _lib.load()
        b.m_capacity = int(capacity) if capacity is not None else int(lib.svo_build_pool_bound(b.m_count, b.m_level))
        dev = fragments.device
        b.m_octree_buffer = torch.empty(max(b.m_capacity, 8), dtype=torch.int32, device=dev)
        b.m_workspace = torch.empty(lib.svo_build_workspace_size(b.m_count, b.m_level, b.m_capacity,
                                                                 int(leaf_words or 0)), dtype=torch.uint8, device=dev)
        b.m_result = torch.zeros(OctreeBuilder.RESULT_WORDS, dtype=torch.int32, device=dev)
        return b

    def CmdBuild(self, stream=None) -> None:
        """OctreeBuilder::CmdBuild (src/OctreeBuilder.cpp:142-210), stream-ordered, no host round trip."""
        lib = _lib.load()
        self._info = None
        _lib.check(lib.svo_build_into(_ptr(self.m_fragments), self.m_count, self.m_level, _ptr(self.m_octree_buffer),
                                      self.m_capacity, _ptr(self.m_workspace), self.m_workspace.numel(),
                                      _ptr(self.m_result), _stream(stream)))

    def Reserve(self) -> None:
        """Shrink the node pool to the exact range of the last build (blocking); later CmdBuild calls on
        the same fragments fit it exactly."""
        info = self.GetInfo()
        lib = _lib.load()
        dev = self.m_fragments.device
        self.m_capacity = int(info["range_words"])
        self.m_octree_buffer = torch.empty(max(self.m_capacity, 8), dtype=torch.int32, device=dev)
        self.m_workspace = torch.empty(lib.svo_build_workspace_size(self.m_count, self.m_level, self.m_capacity, 0),
                                       dtype=torch.uint8, device=dev)
        self._info = None

    def GetInfo(self) -> dict:
        """Per-level counters of the last build (blocking read, like Counter::Read)."""
        if self._info is None:
            r = self.m_result.cpu().numpy().view(np.uint32)
            status = int(r[-1])
            if status & 2:
                raise _lib.SvoError(_lib.SVO_ERR_CAPACITY, "octree pool too small for this build")
            if status & 1:
                raise _lib.SvoError(_lib.SVO_ERR_TIMEOUT, "a device-side wait gave up")
            self._info = {"level": int(r[0]), "fragments": int(r[1]), "range_words": int(r[2]), "leaves": int(r[3]),
                          "level_nodes": [int(x) for x in r[4:4 + self.m_level]]}
        return self._info

    def GetOctreeRange(self) -> int:
        """OctreeBuilder::GetOctreeRange (src/OctreeBuilder.cpp:212-214): used bytes = (blocks + 1) * 32."""
        return self.GetInfo()["range_words"] * 4

    def GetOctree(self) -> torch.Tensor:
        return self.m_octree_buffer

    def GetLevel(self) -> int:
        return self.m_level


# ------------------------------------------------------------------------------------------- Octree
class Octree:
    """Octree (src/Octree.hpp:8-34): the node pool a tracer reads, its level and used range."""

    def __init__(self):
        self.m_buffer: torch.Tensor | None = None
        self.m_range = 0  # bytes
        self.m_level = 0

    @staticmethod
    def Create() -> "Octree":
        return Octree()

    def Update(self, builder: OctreeBuilder) -> None:
        """Octree::Update (src/Octree.cpp:22-35); overflow is impossible here (exact pool bound), and a
        failed build raises instead of being logged."""
        self.m_range = builder.GetOctreeRange()
        self.m_buffer = builder.GetOctree()
        self.m_level = builder.GetLevel()

    @staticmethod
    def FromFragments(fragments: torch.Tensor, level: int, stream=None) -> "Octree":
        """One-call build (svo_build_ex) with torch-owned memory."""
        lib = _lib.load()
        alloc = TorchAllocator(fragments.device)
        out = _lib.OctreeC()
        info = _lib.BuildInfo()
        _lib.check(lib.svo_build_ex(_ptr(fragments), int(fragments.numel()), int(level), ctypes.byref(alloc.struct),
                                    ctypes.byref(out), ctypes.byref(info), _stream(stream)))
        o = Octree()
        o.m_buffer = alloc.take(out.words).view(torch.int32)
        o.m_range = int(out.range_words) * 4
        o.m_level = int(level)
        o.info = {"range_words": int(info.range_words), "leaves": int(info.leaves),
                  "level_nodes": [int(info.level_nodes[i]) for i in range(level)]}
        return o

    def Empty(self) -> bool:
        return self.m_buffer is None and getattr(self, "_view", None) is None

    @property
    def device(self) -> torch.device:
        if self.m_buffer is not None:
            return self.m_buffer.device
        return torch.device("cuda", torch.cuda.current_device())

    def GetBuffer(self) -> torch.Tensor:
        return self.m_buffer

    def GetLevel(self) -> int:
        return self.m_level

    def GetRange(self) -> int:
        return self.m_range

    def words(self) -> torch.Tensor:
        if getattr(self, "_view", None) is not None:
            return _copy_from(self._view.words, self.m_range // 4, torch.int32)
        return self.m_buffer[: self.m_range // 4]

    def c_struct(self) -> _lib.OctreeC:
        if getattr(self, "_view", None) is not None:
            return self._view
        return _lib.OctreeC(self.m_buffer.data_ptr(), self.m_buffer.numel(), self.m_range // 4, self.m_level, 0, 0)

    @staticmethod
    def FromView(view: _lib.OctreeC, owner=None) -> "Octree":
        """An Octree over a node pool the engine owns (a batcher's shared pool): words() copies it out."""
        o = Octree()
        o._view = _lib.OctreeC(view.words, view.capacity, view.range_words, view.level, 0, 0)
        o._owner = owner
        o.m_range = int(view.range_words) * 4
        o.m_level = int(view.level)
        return o


# ------------------------------------------------------------------------------------------- OctreeTracer
class OctreeTracer:
    """OctreeTracer (src/OctreeTracer.hpp:13-70) without the graphics pipeline: rays in, hits out in a
    device buffer (32 B per ray, HIT_DTYPE) instead of a swapchain image."""

    def __init__(self):
        self.m_octree: Octree | None = None
        self.m_camera = None
        self.m_width = 0
        self.m_height = 0
        self.fetches: torch.Tensor | None = None

    @staticmethod
    def Create(octree: Octree, camera=None, width: int = 1280, height: int = 720) -> "OctreeTracer":
        t = OctreeTracer()
        t.m_octree, t.m_camera, t.m_width, t.m_height = octree, camera, int(width), int(height)
        return t

    def Resize(self, width: int, height: int) -> None:
        self.m_width, self.m_height = int(width), int(height)

    def _fetch_ptr(self, count_fetches: bool):
        if not count_fetches:
            return ctypes.c_void_p(0)
        if self.fetches is None:
            self.fetches = torch.zeros(1, dtype=torch.int64, device=self.m_octree.device)
        return _ptr(self.fetches)

    def CmdDrawPipeline(self, hits: torch.Tensor | None = None, stream=None, count_fetches: bool = False) -> torch.Tensor:
        """One primary ray per pixel (shader/octree_tracer.frag:23-37); returns the hit buffer."""
        n = self.m_width * self.m_height
        if hits is None:
            hits = torch.empty(n * HIT_DTYPE.itemsize, dtype=torch.uint8, device=self.m_octree.device)
        cam = camera_struct(self.m_camera)
        oc = self.m_octree.c_struct()
        _lib.check(_lib.load().svo_raycast_camera(ctypes.byref(oc), ctypes.byref(cam), self.m_width, self.m_height,
                                                  _ptr(hits), self._fetch_ptr(count_fetches), _stream(stream)))
        return hits

    def CmdDrawPipelineToHost(self, hits_host: torch.Tensor | None = None, hits: torch.Tensor | None = None,
                              stream=None) -> torch.Tensor:
        """CmdDrawPipeline with the image read back to host memory while it is traced (svo_raycast_camera_download:
        the image in row bands, each copied on a second stream as the next is traced).  hits_host: a page-locked
        uint8 tensor of W*H*32 bytes (allocated pinned when None); hits: the device staging buffer.  Returns
        hits_host; its contents are valid once `stream` has reached this point."""
        n = self.m_width * self.m_height
        if hits is None:
            hits = torch.empty(n * HIT_DTYPE.itemsize, dtype=torch.uint8, device=self.m_octree.device)
        if hits_host is None:
            hits_host = torch.empty(n * HIT_DTYPE.itemsize, dtype=torch.uint8).pin_memory()
        if hits_host.device.type != "cpu" or hits_host.numel() * hits_host.element_size() < n * HIT_DTYPE.itemsize:
            raise ValueError("hits_host must be a host tensor of width * height * 32 bytes")
        cam = camera_struct(self.m_camera)
        oc = self.m_octree.c_struct()
        _lib.check(_lib.load().svo_raycast_camera_download(ctypes.byref(oc), ctypes.byref(cam), self.m_width,
                                                           self.m_height, _ptr(hits), _ptr(hits_host),
                                                           ctypes.c_void_p(0), _stream(stream)))
        return hits_host

    def CmdBeamRenderPass(self, beam: torch.Tensor | None = None, stream=None) -> torch.Tensor:
        """OctreeTracer::CmdBeamRenderPass (src/OctreeTracer.cpp:183-211): the beam image, one start distance
        per corner of each 8x8 pixel tile (float32, ((H+7)//8+1) x ((W+7)//8+1))."""
        lib = _lib.load()
        bw, bh = (self.m_width + 7) // 8 + 1, (self.m_height + 7) // 8 + 1
        if beam is None:
            beam = torch.empty((bh, bw), dtype=torch.float32, device=self.m_octree.device)
        cam = camera_struct(self.m_camera)
        oc = self.m_octree.c_struct()
        _lib.check(lib.svo_beam_prepass(ctypes.byref(oc), ctypes.byref(cam), self.m_width, self.m_height, _ptr(beam),
                                        _stream(stream)))
        return beam

    def CmdDrawPipelineBeam(self, beam: torch.Tensor | None = None, hits: torch.Tensor | None = None, stream=None,
                            count_fetches: bool = False) -> torch.Tensor:
        """CmdDrawPipeline with the beam enabled (shader/octree_tracer.frag:27-33); beam None: computed here."""
        n = self.m_width * self.m_height
        if hits is None:
            hits = torch.empty(n * HIT_DTYPE.itemsize, dtype=torch.uint8, device=self.m_octree.device)
        cam = camera_struct(self.m_camera)
        oc = self.m_octree.c_struct()
        _lib.check(_lib.load().svo_raycast_camera_beam(ctypes.byref(oc), ctypes.byref(cam), self.m_width,
                                                       self.m_height, _ptr(beam), _ptr(hits),
                                                       self._fetch_ptr(count_fetches), _stream(stream)))
        return hits

    def Occlude(self, rays: torch.Tensor, out: torch.Tensor | None = None, stream=None) -> torch.Tensor:
        """Octree_RayMarchOcclude per ray (shader/octree.glsl:504-629): int32 tensor, 1 = occluded."""
        n = rays.numel() // RAY_DTYPE.itemsize
        if out is None:
            out = torch.empty(max(n, 1), dtype=torch.int32, device=rays.device)
        oc = self.m_octree.c_struct()
        _lib.check(_lib.load().svo_occlude(ctypes.byref(oc), _ptr(rays), n, _ptr(out), _stream(stream)))
        return out[:n]

    def Trace(self, rays: torch.Tensor, hits: torch.Tensor | None = None, stream=None,
              count_fetches: bool = False) -> torch.Tensor:
        """Octree_RayMarchLeaf for an explicit ray buffer (RAY_DTYPE bytes on the device)."""
        n = rays.numel() // RAY_DTYPE.itemsize
        if hits is None:
            hits = torch.empty(n * HIT_DTYPE.itemsize, dtype=torch.uint8, device=rays.device)
        oc = self.m_octree.c_struct()
        _lib.check(_lib.load().svo_raycast(ctypes.byref(oc), _ptr(rays), n, _ptr(hits), self._fetch_ptr(count_fetches),
                                           _stream(stream)))
        return hits

    @staticmethod
    def Bounce(hits: torch.Tensor, seed: int, rays: torch.Tensor | None = None, stream=None) -> torch.Tensor:
        """One cosine-weighted diffuse bounce ray per hit (misses give a null ray)."""
        n = hits.numel() // HIT_DTYPE.itemsize
        if rays is None:
            rays = torch.empty(n * RAY_DTYPE.itemsize, dtype=torch.uint8, device=hits.device)
        _lib.check(_lib.load().svo_bounce_rays(_ptr(hits), n, seed & 0xFFFFFFFFFFFFFFFF, _ptr(rays), _stream(stream)))
        return rays


# ------------------------------------------------------------------------------------------- path tracer
class EnvironmentMap:
    """EnvironmentMap (src/EnvironmentMap.hpp:10-54): an HDR image on the device with its pdf weights and
    alias table.  Reset takes the decoded float image (the reference decodes .exr / .hdr files with
    tinyexr / stb_image, which are not part of the engine)."""

    def __init__(self):
        self.m_rotation = 0.0
        self.m_multiplier = 1.0
        self._h = ctypes.c_void_p(0)
        self.width = self.height = 0

    @staticmethod
    def Create() -> "EnvironmentMap":
        return EnvironmentMap()

    def Reset(self, rgba: np.ndarray | None = None) -> None:
        """Reset() empties the map; Reset(image) loads an (h, w, 3|4) float image."""
        lib = _lib.load()
        if self._h:
            lib.svo_envmap_destroy(self._h)
            self._h = ctypes.c_void_p(0)
            self.width = self.height = 0
        if rgba is None:
            return
        img = np.asarray(rgba, np.float32)
        if img.ndim != 3 or img.shape[2] not in (3, 4):
            raise ValueError("environment map must be (h, w, 3) or (h, w, 4)")
        if img.shape[2] == 3:
            img = np.concatenate([img, np.ones(img.shape[:2] + (1,), np.float32)], axis=2)
        img = np.ascontiguousarray(img)
        h = ctypes.c_void_p(0)
        _lib.check(lib.svo_envmap_create(img.ctypes.data_as(ctypes.c_void_p), img.shape[1], img.shape[0],
                                         ctypes.byref(h)))
        self._h, self.height, self.width = h, img.shape[0], img.shape[1]

    def Empty(self) -> bool:
        return not self._h

    def GetTables(self) -> tuple[np.ndarray, np.ndarray]:
        """(texels (h, w, 4) with the pdf weight in alpha, alias table (h, w, 2) uint32)."""
        tex = np.zeros((self.height, self.width, 4), np.float32)
        alias = np.zeros((self.height, self.width, 2), np.uint32)
        _lib.check(_lib.load().svo_envmap_tables(self._h, tex.ctypes.data_as(ctypes.c_void_p),
                                                 alias.ctypes.data_as(ctypes.c_void_p)))
        return tex, alias

    def __del__(self):
        try:
            if self._h:
                _lib.load().svo_envmap_destroy(self._h)
        except Exception:
            pass


class Lighting:
    """Lighting (src/Lighting.hpp:7-20): a constant colour or the environment map."""

    kConstantColor = 0
    kEnvironmentMap = 1

    def __init__(self, environment_map: EnvironmentMap | None = None):
        self.m_light_type = Lighting.kConstantColor
        self.m_sun_radiance = [5.0, 5.0, 5.0]  # kDefaultConstantColor
        self.m_environment_map = environment_map if environment_map is not None else EnvironmentMap.Create()

    @staticmethod
    def Create(environment_map: EnvironmentMap | None = None) -> "Lighting":
        return Lighting(environment_map)

    def GetEnvironmentMapPtr(self) -> EnvironmentMap:
        return self.m_environment_map

    def GetFinalLightType(self) -> int:
        if self.m_light_type == Lighting.kEnvironmentMap and self.m_environment_map.Empty():
            return Lighting.kConstantColor
        return self.m_light_type

    def c_struct(self) -> _lib.LightingC:
        e = self.m_environment_map
        return _lib.LightingC(self.GetFinalLightType(), (ctypes.c_float * 3)(*self.m_sun_radiance),
                              float(e.m_rotation), float(e.m_multiplier), e._h if not e.Empty() else None)


class PathTracer:
    """PathTracer (src/PathTracer.hpp:15-75): progressive path tracing of an octree, the whole path of a
    pixel sample in one kernel (shader/path_tracer.comp), radiance / albedo / normal accumulated on the
    device."""

    kDefaultBounce = 4

    def __init__(self):
        self.m_octree: Octree | None = None
        self.m_camera = None
        self.m_lighting: Lighting | None = None
        self.m_width, self.m_height = 1280, 720  # kDefaultWidth, kDefaultHeight
        self.m_bounce = PathTracer.kDefaultBounce
        self._h = ctypes.c_void_p(0)

    @staticmethod
    def Create(octree: Octree, camera, lighting: Lighting | None = None) -> "PathTracer":
        pt = PathTracer()
        pt.m_octree, pt.m_camera = octree, camera
        pt.m_lighting = lighting if lighting is not None else Lighting.Create()
        return pt

    def Reset(self, stream=None) -> None:
        """Targets of m_width x m_height cleared, Sobol state cleared (m_bounce path vertices)."""
        lib = _lib.load()
        if not self._h:
            h = ctypes.c_void_p(0)
            _lib.check(lib.svo_path_tracer_create(self.m_width, self.m_height, self.m_bounce, ctypes.byref(h)))
            self._h = h
        else:
            _lib.check(lib.svo_path_tracer_reset(self._h, self.m_width, self.m_height, self.m_bounce,
                                                 _stream(stream)))

    def _handle(self):
        if not self._h:
            self.Reset()
        return self._h

    def SetNoise(self, rg: np.ndarray, stream=None) -> None:
        """The 256 x 256 RG8 noise texture (e.g. a blue-noise table)."""
        a = np.ascontiguousarray(rg, np.uint8).reshape(256 * 256 * 2)
        _lib.check(_lib.load().svo_path_tracer_set_noise(self._handle(), a.ctypes.data_as(ctypes.c_void_p),
                                                         _stream(stream)))
        torch.cuda.synchronize()

    def SetSobolMatrices(self, matrices: np.ndarray, stream=None) -> None:
        """Sobol direction numbers, 64 x 32 uint32."""
        a = np.ascontiguousarray(matrices, np.uint32).reshape(64 * 32)
        _lib.check(_lib.load().svo_path_tracer_set_sobol_matrices(self._handle(), a.ctypes.data_as(ctypes.c_void_p),
                                                                  _stream(stream)))
        torch.cuda.synchronize()

    def CmdRender(self, stream=None, samples: int = 1) -> None:
        """PathTracer::CmdRender `samples` times (stream-ordered)."""
        cam = camera_struct(self.m_camera)
        oc = self.m_octree.c_struct()
        light = self.m_lighting.c_struct()
        _lib.check(_lib.load().svo_path_tracer_render(self._handle(), ctypes.byref(oc), ctypes.byref(cam),
                                                      ctypes.byref(light), int(samples), _stream(stream)))

    def GetSPP(self) -> int:
        spp = ctypes.c_uint32(0)
        _lib.check(_lib.load().svo_path_tracer_info(self._handle(), ctypes.byref(spp), None))
        return int(spp.value)

    def GetStatus(self) -> int:
        st = ctypes.c_uint32(0)
        _lib.check(_lib.load().svo_path_tracer_info(self._handle(), None, ctypes.byref(st)))
        return int(st.value)

    def _extract(self, image: int) -> np.ndarray:
        out = np.zeros((self.m_height, self.m_width, 3), np.float32)
        _lib.check(_lib.load().svo_path_tracer_extract(self._handle(), image, out.ctypes.data_as(ctypes.c_void_p),
                                                       _stream()))
        return out

    def ExtractColorImage(self) -> np.ndarray:
        return self._extract(0)

    def ExtractAlbedoImage(self) -> np.ndarray:
        return self._extract(1)

    def ExtractNormalImage(self) -> np.ndarray:
        return self._extract(2)

    def GetImages(self) -> dict:
        """Device copies of the raw targets: color (h, w, 4) float32, albedo / normal (h, w) int32 words,
        sobol (65,) int32."""
        c, a, n, s = (ctypes.c_void_p(0) for _ in range(4))
        _lib.check(_lib.load().svo_path_tracer_images(self._handle(), ctypes.byref(c), ctypes.byref(a),
                                                      ctypes.byref(n), ctypes.byref(s)))
        npx = self.m_width * self.m_height
        dev = self.m_octree.device if self.m_octree is not None else "cuda"
        torch.cuda.synchronize()
        return {"color": _copy_from(c.value, 4 * npx, torch.float32, dev).view(self.m_height, self.m_width, 4),
                "albedo": _copy_from(a.value, npx, torch.int32, dev).view(self.m_height, self.m_width),
                "normal": _copy_from(n.value, npx, torch.int32, dev).view(self.m_height, self.m_width),
                "sobol": _copy_from(s.value, 65, torch.int32, dev)}

    def __del__(self):
        try:
            if self._h:
                _lib.load().svo_path_tracer_destroy(self._h)
        except Exception:
            pass


# ------------------------------------------------------------------------------------------- batches
def _copy_from(ptr: int, count: int, dtype: torch.dtype, device="cuda") -> torch.Tensor:
    """Device copy of `count` elements at an engine-owned device address."""
    out = torch.empty(count, dtype=dtype, device=device)
    if count:
        nbytes = count * out.element_size()
        _lib.check(_lib.load().svo_download(_ptr(out), ctypes.c_void_p(ptr), nbytes, 1, _stream()))
    return out


class BatchBuilder:
    """Many meshes voxelized and built together (svo_batcher): one count pass, one launch per stage for
    all meshes with per-mesh offsets into a shared fragment list and node pool, the launch sequence
    recorded as a CUDA graph and replayed for batches of the same shape.  Per mesh the result equals
    Voxelizer.Create + OctreeBuilder.CmdBuild of that mesh alone."""

    def __init__(self, use_graph: bool = True):
        lib = _lib.load()
        h = ctypes.c_void_p()
        _lib.check(lib.svo_batcher_create(ctypes.byref(h)))
        self.handle = h
        _lib.check(lib.svo_batcher_set_graph(h, 1 if use_graph else 0))
        self._meshes = None
        self._keep = None

    def __del__(self):
        h = getattr(self, "handle", None)
        if h is not None and h.value and _lib._lib is not None:
            _lib._lib.svo_batcher_destroy(h)
            self.handle = None

    def Build(self, meshes, stream=None) -> None:
        """meshes: sequence of (triangles, level), triangles a device tensor of TRIANGLE_DTYPE bytes (or a
        numpy array, uploaded first)."""
        tris = [to_device(np.asarray(t, TRIANGLE_DTYPE)) if isinstance(t, np.ndarray) else t for t, _ in meshes]
        arr = (_lib.BatchMesh * len(tris))()
        for i, (t, (_, level)) in enumerate(zip(tris, meshes)):
            arr[i].tris = t.data_ptr() if t.numel() else 0
            arr[i].n_tris = t.numel() // TRIANGLE_DTYPE.itemsize
            arr[i].level = int(level)
        self._keep = tris
        _lib.check(_lib.load().svo_batcher_build(self.handle, arr, len(tris), _stream(stream)))
        self._meshes = len(tris)

    def __len__(self) -> int:
        return int(_lib.load().svo_batcher_meshes(self.handle))

    def result(self, i: int):
        f, o, info = _lib.Fraglist(), _lib.OctreeC(), _lib.BuildInfo()
        _lib.check(_lib.load().svo_batcher_result(self.handle, i, ctypes.byref(f), ctypes.byref(o), ctypes.byref(info)))
        return f, o, info

    def GetVoxelFragmentList(self, i: int) -> torch.Tensor:
        f, _, _ = self.result(i)
        return _copy_from(f.data or 0, int(f.count), torch.int64)

    def GetOctree(self, i: int) -> Octree:
        _, o, _ = self.result(i)
        return Octree.FromView(o, owner=self)

    def GetInfo(self, i: int) -> dict:
        _, _, info = self.result(i)
        return {"level": int(info.level), "fragments": int(info.fragments), "range_words": int(info.range_words),
                "leaves": int(info.leaves), "level_nodes": [int(info.level_nodes[k]) for k in range(int(info.level))]}

    def stats(self) -> dict:
        c, r = _lib.u64(), _lib.u64()
        _lib.load().svo_batcher_stats(self.handle, ctypes.byref(c), ctypes.byref(r))
        return {"graph_captures": int(c.value), "graph_replays": int(r.value)}


# ------------------------------------------------------------------------------------------- serving
class Server:
    """Resident octrees and continuous batching of trace and rebuild requests (svo_server).  Requests are
    submitted from any thread and complete asynchronously; Wait() returns their timings."""

    def __init__(self, hbm_budget_bytes: int = 0, lanes: int = 0, max_batch_rays: int = 0,
                 max_batch_requests: int = 0, count_fetches: bool = False):
        lib = _lib.load()
        cfg = _lib.ServerConfig(hbm_budget_bytes, lanes, max_batch_rays, max_batch_requests,
                                _lib.SVO_SERVER_COUNT_FETCHES if count_fetches else 0)
        h = ctypes.c_void_p()
        _lib.check(lib.svo_server_create(ctypes.byref(cfg), ctypes.byref(h)))
        self.handle = h
        self._keep: dict[int, object] = {}  # host/device buffers a request reads or writes until it completes

    def close(self) -> None:
        h = getattr(self, "handle", None)
        if h is not None and h.value and _lib._lib is not None:
            _lib._lib.svo_server_destroy(h)
        self.handle = None
        self._keep.clear()

    def __del__(self):
        self.close()

    def BuildScene(self, triangles, level: int) -> int:
        t = to_device(np.asarray(triangles, TRIANGLE_DTYPE)) if isinstance(triangles, np.ndarray) else triangles
        sid = _lib.u32()
        _lib.check(_lib.load().svo_server_build_scene(self.handle, _ptr(t), t.numel() // TRIANGLE_DTYPE.itemsize,
                                                      int(level), ctypes.byref(sid)))
        return int(sid.value)

    def AddOctree(self, octree: Octree) -> int:
        oc = octree.c_struct()
        sid = _lib.u32()
        _lib.check(_lib.load().svo_server_add_octree(self.handle, ctypes.byref(oc), ctypes.byref(sid)))
        self._keep[-1 - int(sid.value)] = octree
        return int(sid.value)

    def Scene(self, scene: int) -> Octree:
        o = _lib.OctreeC()
        _lib.check(_lib.load().svo_server_scene(self.handle, scene, ctypes.byref(o)))
        return Octree.FromView(o, owner=self)

    def SubmitCamera(self, scene: int, camera, width: int, height: int, n_primary: int, seed: int,
                     hits_host: torch.Tensor) -> int:
        """Camera request: hits_host (pinned uint8 tensor) receives 2 * n_primary hits."""
        r = _lib.TraceRequest()
        r.scene, r.mode = scene, _lib.SVO_REQUEST_CAMERA
        r.camera = camera_struct(camera)
        r.width, r.height, r.n_primary = width, height, n_primary
        r.hits = hits_host.data_ptr()
        r.seed = seed & 0xFFFFFFFFFFFFFFFF
        t = _lib.u64()
        _lib.check(_lib.load().svo_server_submit_trace(self.handle, ctypes.byref(r), ctypes.byref(t)))
        self._keep[int(t.value)] = hits_host
        return int(t.value)

    def SubmitRays(self, scene: int, rays_host: torch.Tensor, hits_host: torch.Tensor) -> int:
        r = _lib.TraceRequest()
        r.scene, r.mode = scene, _lib.SVO_REQUEST_RAYS
        r.n_rays = rays_host.numel() // RAY_DTYPE.itemsize
        r.rays, r.hits = rays_host.data_ptr(), hits_host.data_ptr()
        t = _lib.u64()
        _lib.check(_lib.load().svo_server_submit_trace(self.handle, ctypes.byref(r), ctypes.byref(t)))
        self._keep[int(t.value)] = (rays_host, hits_host)
        return int(t.value)

    def SubmitRebuild(self, scene: int, triangles: torch.Tensor, level: int) -> int:
        t = _lib.u64()
        _lib.check(_lib.load().svo_server_submit_rebuild(self.handle, scene, _ptr(triangles),
                                                         triangles.numel() // TRIANGLE_DTYPE.itemsize, int(level),
                                                         ctypes.byref(t)))
        self._keep[int(t.value)] = triangles
        return int(t.value)

    def Wait(self, ticket: int, timeout_ms: int = -1) -> dict:
        res = _lib.RequestResult()
        code = _lib.load().svo_server_wait(self.handle, ticket, timeout_ms, ctypes.byref(res))
        if code == _lib.SVO_ERR_TIMEOUT:  # still running: keep its buffers
            _lib.check(code)
        self._keep.pop(ticket, None)
        _lib.check(code)
        return {"status": int(res.status), "batch_requests": int(res.batch_requests), "submit_us": res.submit_us,
                "launch_us": res.launch_us, "done_us": res.done_us}

    def stats(self) -> dict:
        st = _lib.ServerStats()
        _lib.load().svo_server_get_stats(self.handle, ctypes.byref(st))
        return {name: int(getattr(st, name)) for name, _ in _lib.ServerStats._fields_}


# ------------------------------------------------------------------------------------------- files
def load_obj(path: str) -> np.ndarray:
    """Scene::load_meshes for the engine (svo_load_obj): triangles (TRIANGLE_DTYPE) in [0,1]^3 with the
    reference's normalisation and per-material albedo."""
    lib = _lib.load()
    ptr, n = ctypes.c_void_p(), _lib.u32()
    _lib.check(lib.svo_load_obj(path.encode(), ctypes.byref(ptr), ctypes.byref(n)))
    try:
        raw = ctypes.string_at(ptr, n.value * TRIANGLE_DTYPE.itemsize)
    finally:
        lib.svo_free_host(ptr)
    return np.frombuffer(raw, TRIANGLE_DTYPE).copy()


def write_octree_file(words: np.ndarray, level: int, path: str) -> None:
    w = np.ascontiguousarray(words, np.uint32)
    _lib.check(_lib.load().svo_octree_write_host(w.ctypes.data_as(ctypes.c_void_p), len(w), int(level), path.encode()))


def read_octree_file(path: str) -> tuple[np.ndarray, int]:
    lib = _lib.load()
    ptr, rng, lvl = ctypes.c_void_p(), _lib.u32(), _lib.u32()
    _lib.check(lib.svo_octree_read_host(path.encode(), ctypes.byref(ptr), ctypes.byref(rng), ctypes.byref(lvl)))
    try:
        words = np.frombuffer(ctypes.string_at(ptr, rng.value * 4), np.uint32).copy()
    finally:
        lib.svo_free_host(ptr)
    return words, int(lvl.value)


class _OwnedPool:
    """A library-owned device pool (svo_octree_load) released with svo_octree_destroy."""

    def __init__(self, oc: _lib.OctreeC):
        self.oc = oc

    def __del__(self):
        if _lib._lib is not None and self.oc.words:
            _lib._lib.svo_octree_destroy(ctypes.byref(self.oc), None)


def save_octree(octree: Octree, path: str, stream=None) -> None:
    oc = octree.c_struct()
    _lib.check(_lib.load().svo_octree_save(ctypes.byref(oc), path.encode(), _stream(stream)))


def load_octree(path: str, stream=None) -> Octree:
    oc = _lib.OctreeC()
    _lib.check(_lib.load().svo_octree_load(path.encode(), ctypes.byref(oc), _stream(stream)))
    return Octree.FromView(oc, owner=_OwnedPool(oc))


# ------------------------------------------------------------------------------------------- textures
UV_DTYPE = np.dtype([("uv", "<f4", (6,)), ("texture", "<u4"), ("reserved", "<u4")])


class TextureSet:
    """The scene's textures (Scene::load_textures, src/Scene.cpp:225-309, minus the file decoding): RGBA8
    images with sRGB colour and linear alpha; mip chains built on the host, texels on the device."""

    def __init__(self, images):
        imgs = [np.ascontiguousarray(i, np.uint8) for i in images]
        for i in imgs:
            if i.ndim != 3 or i.shape[2] != 4:
                raise ValueError("textures must be (h, w, 4) uint8")
        ptrs = (ctypes.c_void_p * max(1, len(imgs)))(*[i.ctypes.data for i in imgs])
        ws = np.array([i.shape[1] for i in imgs] + [0], np.uint32)
        hs = np.array([i.shape[0] for i in imgs] + [0], np.uint32)
        h = ctypes.c_void_p(0)
        _lib.check(_lib.load().svo_texture_set_create(ptrs, ws.ctypes.data_as(ctypes.c_void_p),
                                                      hs.ctypes.data_as(ctypes.c_void_p), len(imgs), ctypes.byref(h)))
        self._h, self.count = h, len(imgs)

    def GetLevel(self, texture: int, level: int) -> np.ndarray:
        w, h = ctypes.c_uint32(0), ctypes.c_uint32(0)
        lib = _lib.load()
        _lib.check(lib.svo_texture_set_level(self._h, texture, level, None, ctypes.byref(w), ctypes.byref(h)))
        out = np.zeros((h.value, w.value, 4), np.uint8)
        _lib.check(lib.svo_texture_set_level(self._h, texture, level, out.ctypes.data_as(ctypes.c_void_p), None, None))
        return out

    def __del__(self):
        try:
            if self._h:
                _lib.load().svo_texture_set_destroy(self._h)
        except Exception:
            pass


def voxelize_textured(triangles, uvs, level: int, textures: TextureSet | None, stream=None) -> torch.Tensor:
    """Voxelizer with texture-sampled fragment colour and the alpha discard (shader/voxelizer.frag:27-36):
    uvs[i] (UV_DTYPE) belongs to triangles[i]; returns the surviving fragments (int64 tensor)."""
    tris = triangles if isinstance(triangles, torch.Tensor) else to_device(np.asarray(triangles, TRIANGLE_DTYPE))
    uv = uvs if isinstance(uvs, torch.Tensor) else to_device(np.asarray(uvs, UV_DTYPE))
    n = tris.numel() // TRIANGLE_DTYPE.itemsize
    fl = _lib.Fraglist()
    _lib.check(_lib.load().svo_voxelize_textured(_ptr(tris), _ptr(uv), n, level,
                                                 textures._h if textures is not None else None, ctypes.byref(fl),
                                                 _stream(stream)))
    out = _copy_from(fl.data, fl.count, torch.int64, tris.device)
    _lib.load().svo_fraglist_destroy(ctypes.byref(fl), _stream(stream))
    return out


# ------------------------------------------------------------------------------------------- functional
def voxelize(triangles, level: int, stream=None) -> torch.Tensor:
    return Voxelizer.Create(triangles, level, stream).GetVoxelFragmentList()


def build(fragments: torch.Tensor, level: int, stream=None) -> Octree:
    return Octree.FromFragments(fragments, level, stream)


def raycast(octree: Octree, rays: torch.Tensor, stream=None) -> torch.Tensor:
    return OctreeTracer.Create(octree).Trace(rays, stream=stream)


def hits_numpy(hits: torch.Tensor) -> np.ndarray:
    return from_device(hits, HIT_DTYPE)
