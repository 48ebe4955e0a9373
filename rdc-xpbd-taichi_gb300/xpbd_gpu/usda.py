"""Time-sampled USD export of the solver's mesh without pxr (ASCII ``.usda``).

The reference exports through ``pxr`` (``utils/renderer.py:8-122``,
``usd_export.py:58-92``): a root Xform, one Mesh whose ``points`` carry a time
sample per rendered frame, and static Sphere / Cube / plane-Mesh prims for the
SDFs.  ``USDMeshRenderer`` here has the same constructor and methods
(``add_dynamic_mesh``, ``add_static_sphere``, ``add_static_cube``,
``add_static_plane``, ``render``, ``save``, ``get_root_prim_path``,
``get_file_size_mb``) and writes the same prims as USD's ASCII layer format,
which USD tools read like the binary one (a binary crate file needs pxr, so
``use_binary`` writes ASCII too).

Frame data leaves the GPU asynchronously: ``render`` exports the positions
into a device staging tensor, copies them into one of a few pinned host
buffers with ``non_blocking`` on the current stream and records an event; a
writer thread waits for the event, formats the frame and appends it to a
spool file, so formatting overlaps the next frames' simulation.  ``save``
assembles the layer from the header, the prims and the spooled samples.
"""
import os
import queue
import tempfile
import threading

import numpy as np


def _fmt_points(p):
    """USD text of a point3f[] value: [(x, y, z), ...] with 9 significant digits."""
    p = np.asarray(p, dtype=np.float64).reshape(-1, 3)
    if len(p) == 0:
        return "[]"
    body = ", ".join("(%.9g, %.9g, %.9g)" % tuple(r) for r in p.tolist())
    return "[" + body + "]"


def _fmt_ints(a):
    return "[" + ", ".join(str(int(v)) for v in np.asarray(a).reshape(-1).tolist()) + "]"


def _fmt3(v):
    v = np.asarray(v, dtype=np.float64).reshape(3)
    return "(%.9g, %.9g, %.9g)" % tuple(v.tolist())


def _device_source(vert):
    """(solver, field id) when `vert` is a device-backed vertex field of this
    package (``mesh.verts.x``), else None."""
    s, fid = getattr(vert, "_s", None), getattr(vert, "_id", None)
    if s is not None and fid is not None and hasattr(s, "_export_vec3_device"):
        return s, fid
    return None


class USDMeshRenderer:
    """Drop-in for the reference's ``utils.renderer.USDMeshRenderer``."""

    def __init__(self, filepath, totalframes, fps, use_binary=True, enable_streaming=False, stream_chunk_size=100,
                 root_prim_path="/root", pinned_buffers=3):
        if filepath.endswith(".usdc"):
            filepath = filepath[:-5] + ".usda"
        self.filepath = filepath
        self.totalframes = int(totalframes)
        self.fps = fps
        self.frame = 0
        self.time = 0.0
        self.enable_streaming = enable_streaming
        self.stream_chunk_size = stream_chunk_size
        self.root_prim_path = root_prim_path if root_prim_path.startswith("/") else "/" + root_prim_path
        self._static = []      # text of static prims
        self._meshes = []      # (name, vert field, faces, default points)
        self._spools = []      # one temp file per dynamic mesh
        self._queue = queue.Queue()
        self._free = queue.Queue()
        self._n_pinned = int(pinned_buffers)
        self._pinned = None
        self._error = None
        self._thread = None

    # -- prims ------------------------------------------------------------------
    def get_root_prim_path(self):
        return self.root_prim_path

    def add_static_sphere(self, center, radius, name="sdf_sphere"):
        self._static.append('    def Sphere "%s"\n    {\n        double radius = %.9g\n'
                            '        double3 xformOp:translate = %s\n'
                            '        uniform token[] xformOpOrder = ["xformOp:translate"]\n    }\n'
                            % (name, float(radius), _fmt3(center)))

    def add_static_cube(self, center, size, name="sdf_cube"):
        self._static.append('    def Cube "%s"\n    {\n        float3 xformOp:scale = %s\n'
                            '        double3 xformOp:translate = %s\n'
                            '        uniform token[] xformOpOrder = ["xformOp:scale", "xformOp:translate"]\n    }\n'
                            % (name, _fmt3(size), _fmt3(center)))

    def add_static_plane(self, point, normal, extent=2.0, name="sdf_plane"):
        """A two-triangle square of side `extent` centred at `point`, normal `normal`
        (the construction of utils/renderer.py:64-101)."""
        n = np.asarray(normal, dtype=np.float32)
        nn = np.linalg.norm(n)
        n = np.array([0.0, 1.0, 0.0], dtype=np.float32) if nn < 1e-8 else n / nn
        ref = np.array([1.0, 0.0, 0.0], dtype=np.float32)
        if abs(np.dot(ref, n)) > 0.9:
            ref = np.array([0.0, 0.0, 1.0], dtype=np.float32)
        u = np.cross(n, ref)
        u = u / max(np.linalg.norm(u), 1e-8)
        v = np.cross(n, u)
        p = np.asarray(point, dtype=np.float32)
        h = float(extent) * 0.5
        pts = np.array([p - h * u - h * v, p - h * u + h * v, p + h * u + h * v, p + h * u - h * v], dtype=np.float32)
        self._static.append('    def Mesh "%s"\n    {\n        int[] faceVertexCounts = [3, 3]\n'
                            '        int[] faceVertexIndices = [0, 1, 2, 0, 2, 3]\n'
                            '        point3f[] points = %s\n'
                            '        uniform token subdivisionScheme = "none"\n    }\n' % (name, _fmt_points(pts)))

    def add_dynamic_mesh(self, vert, face, meshname="mesh"):
        faces = np.asarray(face.to_numpy() if hasattr(face, "to_numpy") else face).reshape(-1)
        self._meshes.append((meshname, vert, faces, np.asarray(vert.to_numpy())))
        fd, path = tempfile.mkstemp(prefix="xpbd_usda_", suffix=".spool")
        self._spools.append((os.fdopen(fd, "w"), path))

    # -- frames -----------------------------------------------------------------
    def _writer(self):
        while True:
            item = self._queue.get()
            if item is None:
                return
            k, t, buf, ev = item
            try:
                if ev is not None:
                    ev.synchronize()
                arr = buf.numpy() if hasattr(buf, "numpy") else buf
                self._spools[k][0].write("            %d: %s,\n" % (t, _fmt_points(arr)))
            except Exception as e:  # reported by save()
                self._error = e
            finally:
                if ev is not None:
                    self._free.put((k, buf))

    def _start(self):
        if self._thread is None:
            self._thread = threading.Thread(target=self._writer, daemon=True)
            self._thread.start()

    def _pinned_buffer(self, k, n):
        import torch
        if self._pinned is None:
            self._pinned = True
            for kk, (_, _, _, pts) in enumerate(self._meshes):
                for _ in range(self._n_pinned):
                    self._free.put((kk, torch.empty((len(pts), 3), dtype=torch.float32).pin_memory()))
        held = []
        while True:
            kk, buf = self._free.get()
            if kk == k:
                for h in held:
                    self._free.put(h)
                return buf
            held.append((kk, buf))

    def render(self):
        """Record the current positions of every dynamic mesh at time code frame + 1."""
        if self.frame >= self.totalframes:
            return
        self._start()
        t = self.frame + 1
        for k, (_, vert, _, pts) in enumerate(self._meshes):
            src = _device_source(vert)
            if src is None:
                self._queue.put((k, t, np.asarray(vert.to_numpy()), None))
                continue
            import torch
            solver, fid = src
            dev = solver._export_vec3_device(fid)
            buf = self._pinned_buffer(k, len(pts))
            buf.copy_(dev, non_blocking=True)
            ev = torch.cuda.Event()
            ev.record()
            self._queue.put((k, t, buf, ev))
        self.frame += 1
        self.time = self.frame / self.fps
        if self.enable_streaming and self.frame % self.stream_chunk_size == 0:
            self.save()

    # -- output -----------------------------------------------------------------
    def _drain(self):
        if self._thread is not None:
            self._queue.put(None)
            self._thread.join()
            self._thread = None
        if self._error is not None:
            raise RuntimeError("USD export failed: %s" % self._error)

    def save(self):
        """Write the layer: header, root Xform, meshes with their time samples so far, SDF prims."""
        self._drain()
        root = self.root_prim_path.strip("/").split("/")[-1] or "root"
        tmp = self.filepath + ".tmp"
        d = os.path.dirname(self.filepath)
        if d:
            os.makedirs(d, exist_ok=True)
        with open(tmp, "w") as out:
            out.write('#usda 1.0\n(\n    defaultPrim = "%s"\n    endTimeCode = %d\n    startTimeCode = 1\n'
                      '    timeCodesPerSecond = %s\n    upAxis = "Y"\n)\n\n' % (root, self.totalframes, self.fps))
            out.write('def Xform "%s"\n{\n' % root)
            for (name, _, faces, pts), (spool, path) in zip(self._meshes, self._spools):
                spool.flush()
                out.write('    def Mesh "%s"\n    {\n' % name)
                out.write('        int[] faceVertexCounts = %s\n' % _fmt_ints(np.full(len(faces) // 3, 3)))
                out.write('        int[] faceVertexIndices = %s\n' % _fmt_ints(faces))
                out.write('        point3f[] points = %s\n' % _fmt_points(pts))
                out.write('        point3f[] points.timeSamples = {\n')
                with open(path) as f:
                    for line in f:
                        out.write(line)
                out.write('        }\n        uniform token subdivisionScheme = "none"\n    }\n')
            for prim in self._static:
                out.write(prim)
            out.write('}\n')
        os.replace(tmp, self.filepath)

    def get_file_size_mb(self):
        return os.path.getsize(self.filepath) / (1024 * 1024) if os.path.exists(self.filepath) else 0.0

    def close(self):
        self._drain()
        for spool, path in self._spools:
            spool.close()
            try:
                os.remove(path)
            except OSError:
                pass
        self._spools = []

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def read_usda_points(path, mesh="deformable_mesh"):
    """Time samples of `mesh`'s points in a layer written by USDMeshRenderer:
    {time code: (N, 3) float64}.  A reader for this writer's own layout (tests)."""
    import re
    text = open(path).read()
    m = re.search(r'def Mesh "%s"\s*\{(.*?)\n    \}' % re.escape(mesh), text, re.S)
    if not m:
        raise KeyError(mesh)
    block = m.group(1)
    ts = re.search(r"points\.timeSamples = \{\n(.*?)\n\s*\}", block, re.S)
    out = {}
    if ts:
        for line in ts.group(1).splitlines():
            t, rest = line.strip().split(":", 1)
            nums = [float(x) for x in re.findall(r"[-+0-9.eEinfa]+", rest)]
            out[int(t)] = np.asarray(nums, dtype=np.float64).reshape(-1, 3)
    return out


def add_sdfs(renderer, sdf_config):
    """The SDF prims of usd_export.py:63-95: one prim per SDF, named by kind and
    list index, read through the SDF objects' [None]-indexable parameters."""
    from xpbd_gpu.sdf import CubeSdf, PlaneSdf, SphereSdf
    items = list(enumerate(sdf_config)) if isinstance(sdf_config, (list, tuple)) else [(None, sdf_config)]
    for i, s in items:
        suffix = "" if i is None else "_%d" % i
        if isinstance(s, SphereSdf):
            renderer.add_static_sphere(center=s.center[None].to_numpy(), radius=float(s.radius[None]),
                                       name="sdf_sphere" + suffix)
        elif isinstance(s, CubeSdf):
            renderer.add_static_cube(center=s.center[None].to_numpy(),
                                     size=(s.half_size[None].to_numpy() * 2.0).astype(np.float32),
                                     name="sdf_cube" + suffix)
        elif isinstance(s, PlaneSdf):
            renderer.add_static_plane(point=s.point[None].to_numpy(), normal=s.dir[None].to_numpy(), extent=4.0,
                                      name="sdf_plane" + suffix)
