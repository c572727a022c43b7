"""Scene and TriangleRaster: Tina's top-level API (tina/scene/raster.py,
tina/core/triangle.py) over the CUDA library.

`Scene.render()` issues one t3_render call per frame: scene upload, depth-key
clear, the rasteriser over every object, then deferred shading with the ACES
epilogue.  All buffers are torch tensors on the CUDA device; `scene.img` is a
float32 tensor of shape (W, H, 3) indexed [x, y] like Tina's Taichi field.
"""
import ctypes as C

import numpy as np
import torch

from . import _native as N
from ._device import default_device, require_cuda
from .engine import Engine
from .lighting import Lighting
from .materials import Diffuse, compile_material

_UNSUPPORTED_OPTIONS = ('ssr', 'ssao')
RASTER_MODES = {'direct': N.T3_RASTER_DIRECT, 'binned': N.T3_RASTER_BINNED}


class _Obj:
    def __init__(self, material, raster):
        self.material = material
        self.raster = raster


def _stream():
    return torch.cuda.current_stream().cuda_stream


class _KeyRaster:
    """The rasteriser protocol set_object / render_occup / render_color
    (tina/scene/raster.py:183-187) over the engine's packed depth-key buffer.

    Engine.clear_depth empties the frame's keys once per frame
    (tina/scene/raster.py:177); each render_occup depth-tests the current
    object against them without clearing them (tina/core/triangle.py:121-125),
    its faces numbered after the objects rasterised before it in the frame, so
    an earlier object keeps a pixel on a depth tie (the strict `>` of
    triangle.py:123); engine.depth then holds the frame's int32 depths.
    render_color shades only the pixels this object won (occup != -1,
    triangle.py:134-139), leaving every other pixel of the image as it is."""

    mesh = None
    _base = 0
    _nfaces = 0

    def flags(self, tonemap=False):
        return N.T3_TONEMAP if tonemap else 0

    def _fill_frame(self, fr):
        pass

    # -- protocol ---------------------------------------------------------
    def set_object(self, mesh):
        mesh.pre_compute()
        self.check_faces(mesh)
        self.mesh = mesh

    def render_occup(self):
        """Rasterises the current object into the engine's depth keys."""
        require_cuda(type(self).__name__ + '.render_occup')
        lib = N.load()
        dev = default_device()
        eng = self.engine
        if eng.keys is None or eng.keys.numel() != eng.res[0] * eng.res[1]:
            eng.clear_depth()
        keep = []
        ob = N.t3_object()
        self.mesh._t3_fill(ob.mesh, dev, keep)
        self._nfaces = ob.nfaces = self.check_faces(self.mesh)
        self._base = ob.face_base = eng._claim_faces(ob.nfaces)
        fr = N.t3_frame()
        eng._t3_fill_frame(fr, self.flags(), 0.0)
        self._fill_frame(fr)
        need = 256 + 4 * max(1, ob.nfaces)
        ws = getattr(self, '_ws', None)
        if ws is None or ws.numel() < need:
            self._ws = ws = torch.empty(need, dtype=torch.uint8, device=dev)
            self._status = torch.zeros(1, dtype=torch.int32, device=dev)
        N.check(lib.t3_raster(C.byref(fr), C.byref(ob), eng.keys.data_ptr(), ws.data_ptr(), ws.numel(),
                              self._status.data_ptr(), _stream()), 't3_raster')
        self._keep = keep
        eng._keys_to_depth()

    @property
    def occup(self):
        """This object's winning face per pixel, -1 elsewhere (TriangleRaster.occup)."""
        ids = (self.engine.keys & 0xFFFFFFFF) - self._base
        mine = (self.engine.keys != -1) & (ids >= 0) & (ids < self._nfaces)
        return torch.where(mine, ids, torch.full_like(ids, -1)).to(torch.int32)

    def render_color(self, shader):
        """Shades the pixels this object won with `shader` (a Shader of the scene)."""
        shader.shade_from_keys(self, self.engine.keys)


class TriangleRaster(_KeyRaster):
    """TriangleRaster (tina/core/triangle.py:5-153) with the protocol of
    _KeyRaster.  Options: maxfaces, smoothing, texturing, culling (default
    True), clipping (default True)."""

    def __init__(self, engine, maxfaces=None, smoothing=False, texturing=False, culling=True,
                 clipping=True, **extra_options):
        self.engine = engine
        self.res = engine.res
        self.maxfaces = maxfaces
        self.smoothing = smoothing
        self.texturing = texturing
        self.culling = culling
        self.clipping = clipping

    def flags(self, tonemap=False):
        f = 0
        f |= N.T3_CULLING if self.culling else 0
        f |= N.T3_CLIPPING if self.clipping else 0
        f |= N.T3_SMOOTHING if self.smoothing else 0
        f |= N.T3_TEXTURING if self.texturing else 0
        f |= N.T3_TONEMAP if tonemap else 0
        return f

    def check_faces(self, mesh):
        n = mesh.get_nfaces()
        if self.maxfaces is not None and n > self.maxfaces:
            raise ValueError(f'mesh has {n} faces, more than maxfaces={self.maxfaces}')
        return n


class ParticleRaster(_KeyRaster):
    """ParticleRaster (tina/core/particle.py): particles rasterised as shaded
    spheres into the same depth keys as the triangles.  Options kept: maxpars,
    coloring, clipping."""

    def __init__(self, engine, maxpars=None, coloring=True, clipping=True, **extra_options):
        self.engine = engine
        self.res = engine.res
        self.maxpars = maxpars
        self.coloring = coloring
        self.clipping = clipping

    def flags(self, tonemap=False):
        return (N.T3_CLIPPING if self.clipping else 0) | (N.T3_TONEMAP if tonemap else 0)

    def check_faces(self, pars):
        n = pars.get_npars()
        if self.maxpars is not None and n > self.maxpars:
            raise ValueError(f'{n} particles, more than maxpars={self.maxpars}')
        return n


class WireframeRaster(_KeyRaster):
    """WireframeRaster (tina/core/wireframe.py): each line is walked one pixel
    per step along its major axis (draw_line), with the depth interpolated
    perspective-correctly between the endpoints, through the same depth keys
    as the triangles; a pixel a line wins takes the raster's line colour.
    Options kept: maxwires, linewidth (stored: the reference draws one-pixel
    lines whatever its value), linecolor, clipping (default False: a line is
    dropped only when both endpoints leave the clip cube)."""

    def __init__(self, engine, maxwires=None, linewidth=1.5, linecolor=(.9, .6, 0), clipping=False,
                 **extra_options):
        self.engine = engine
        self.res = engine.res
        self.maxwires = maxwires
        self.linewidth = linewidth
        self.linecolor = tuple(float(c) for c in np.broadcast_to(np.asarray(linecolor, np.float32), (3,)))
        self.clipping = clipping

    def check_faces(self, mesh):
        n = mesh.get_nfaces()
        if self.maxwires is not None and n > self.maxwires:
            raise ValueError(f'{n} lines, more than maxwires={self.maxwires}')
        return n

    def _t3_fill(self, fr):
        for k in range(3):
            fr.linecolor[k] = self.linecolor[k]
        if self.clipping:
            fr.flags |= N.T3_WIRE_CLIPPING

    _fill_frame = _t3_fill


class Shader:
    """Shader(img, lighting, material) (tina/core/shader.py:112-135): shades the
    winning fragments of one raster into `img`.  `outputs` (optional) names
    more buffers written at the same pixels: 'face_id' (global face id),
    'depth_f' (float depth)."""

    def __init__(self, img, lighting, material, outputs=None):
        self.img = img
        self.lighting = lighting
        self.material = material
        self.outputs = outputs or {}
        self._ws = None

    def _workspace(self, lib, sc, dev):
        size = C.c_size_t()
        N.check(lib.t3_workspace_size(C.byref(sc), N.T3_RASTER_DIRECT, 16, 0, C.byref(size)),
                't3_workspace_size')
        if self._ws is None or self._ws.numel() < size.value:
            self._ws = torch.empty(size.value, dtype=torch.uint8, device=dev)
        return self._ws

    def _describe(self, raster, dev, keep, flags):
        sc = N.t3_scene()
        raster.engine._t3_fill_frame(sc.frame, raster.flags() | flags, getattr(raster, 'bgcolor', 0.0))
        raster._fill_frame(sc.frame)
        self.lighting._t3_fill(sc.lighting)
        if hasattr(self.lighting, '_t3_fill_device'):
            self.lighting._t3_fill_device(sc.lighting, dev, keep)
        return sc

    def shade_from_keys(self, raster, keys):
        """TriangleRaster.render_color: the pixels whose key belongs to the
        raster's current object, shaded in place (nothing else is written)."""
        require_cuda('Shader')
        lib = N.load()
        keep = []
        dev = default_device()
        sc = self._describe(raster, dev, keep, N.T3_SHADE_OWNED)
        sc.nobjects = 1
        ob = sc.objects[0]
        raster.mesh._t3_fill(ob.mesh, dev, keep)
        if isinstance(raster, ParticleRaster) and not raster.coloring:
            ob.mesh.norms = None
        ob.nfaces = raster._nfaces
        ob.face_base = raster._base
        stride = raster.mesh.attr_stride() if hasattr(raster.mesh, 'attr_stride') else 0
        mat, _ = compile_material(self.material, stride, dev, keep)
        ob.material = mat
        self._shade(lib, sc, keys, dev)

    def _shade(self, lib, sc, keys, dev):
        outs = N.t3_outputs()
        outs.rgb = self.img.data_ptr()
        if 'face_id' in self.outputs:
            outs.face_id = self.outputs['face_id'].data_ptr()
        if 'depth_f' in self.outputs:
            outs.depth_f = self.outputs['depth_f'].data_ptr()
        ws = self._workspace(lib, sc, dev)
        N.check(lib.t3_shade(C.byref(sc), keys.data_ptr(), ws.data_ptr(), ws.numel(), C.byref(outs),
                             _stream()), 't3_shade')


class BackgroundShader(Shader):
    """BackgroundShader + Engine.render_background (tina/core/shader.py,
    tina/core/engine.py:42-49): the pixels no fragment reached take the
    background colour, or under SkyboxLighting the sky along the view ray."""

    def __init__(self, img, lighting, bgcolor=0.0, outputs=None):
        super().__init__(img, lighting, None, outputs)
        self.bgcolor = bgcolor

    def shade_empty(self, engine):
        require_cuda('BackgroundShader')
        lib = N.load()
        keep = []
        dev = default_device()
        sc = N.t3_scene()
        engine._t3_fill_frame(sc.frame, N.T3_SHADE_EMPTY, self.bgcolor)
        self.lighting._t3_fill(sc.lighting)
        if hasattr(self.lighting, '_t3_fill_device'):
            self.lighting._t3_fill_device(sc.lighting, dev, keep)
        sc.nobjects = 0
        self._shade(lib, sc, engine.keys, dev)


class Scene:
    """Tina's Scene(res, **options) (tina/scene/raster.py:5-258).

    Options kept from the reference: smoothing, texturing, culling, clipping,
    maxfaces, tonemap (default True), bgcolor (default 0), blooming, fxaa, taa
    (post-processing in the reference's order), ibl (SkyboxLighting).
    Extension options: raster ('direct' | 'binned'), tile (8 | 16 | 32),
    bin_capacity (entries per tile bin, 0 = automatic), check_bins (re-render
    with doubled bins when a bin overflowed; default True).  ssr and ssao are
    outside this rasteriser build.
    """

    def __init__(self, res_x=512, res_y=None, **options):
        for opt in _UNSUPPORTED_OPTIONS:
            if options.get(opt, False):
                raise NotImplementedError(f'Scene({opt}=True) is not part of this rasteriser build')
        self.engine = Engine(res_x, res_y)
        self.res = self.engine.res
        self.options = options
        self.ibl = options.get('ibl', False)
        self.tonemap = options.get('tonemap', True)
        # post-processing (raster.py:72-85, :200-207): blooming on the HDR
        # image, then the tonemap, FXAA, and temporal accumulation
        from .postp import Accumator, Blooming, FXAA, ToneMapping
        self.blooming = Blooming(self.res) if options.get('blooming', False) else None
        self.fxaa = FXAA(self.res) if options.get('fxaa', False) else None
        self.taa = bool(options.get('taa', False))
        self.accum = Accumator(self.res) if self.taa else None
        self._tonemap_pass = ToneMapping(self.res)
        self.bgcolor = options.get('bgcolor', 0)
        self.raster_mode = options.get('raster', 'direct')
        if self.raster_mode not in RASTER_MODES:
            raise ValueError(f"raster must be one of {list(RASTER_MODES)}")
        self.tile = int(options.get('tile', 16))
        self.bin_capacity = int(options.get('bin_capacity', 0))
        # read the device status after each binned frame and grow overflowing bins
        self.check_bins = bool(options.get('check_bins', True))
        if self.ibl:
            from .skybox import SkyboxLighting
            self.lighting = options.get('lighting') or SkyboxLighting()
        else:
            self.lighting = Lighting()
            # add_default_lights (tina/scene/raster.py:89-93)
            self.lighting.add_light(dir=[1, 2, 3], color=[0.9, 0.9, 0.9])
            self.lighting.set_ambient_light([0.1, 0.1, 0.1])
        self.default_material = Diffuse()
        self.materials = []
        self.shaders = {}
        self.objects = {}
        self.raster_options = {k: options[k] for k in
                               ('maxfaces', 'smoothing', 'texturing', 'culling', 'clipping')
                               if k in options}
        self.triangle_raster = None
        self.image = None
        self.face_id = None
        self.depth_f = None
        self._ws = None
        self._status = None
        self._keep = []
        self._last_scene = None

    def add_object(self, object, material=None, raster=None):
        """(tina/scene/raster.py:112-146)"""
        assert object not in self.objects
        if material is None:
            material = self.default_material
        if raster is None:
            if hasattr(object, 'get_nfaces'):
                if hasattr(object, 'get_npolygon') and object.get_npolygon() == 2:
                    if getattr(self, 'wireframe_raster', None) is None:
                        self.wireframe_raster = WireframeRaster(
                            self.engine, **{k: self.options[k] for k in
                                            ('maxwires', 'linewidth', 'linecolor', 'clipping')
                                            if k in self.options})
                    raster = self.wireframe_raster
                else:
                    if self.triangle_raster is None:
                        self.triangle_raster = TriangleRaster(self.engine, **self.raster_options)
                    raster = self.triangle_raster
            elif hasattr(object, 'get_npars'):
                if getattr(self, 'particle_raster', None) is None:
                    self.particle_raster = ParticleRaster(
                        self.engine, **{k: self.options[k] for k in ('maxpars', 'coloring', 'clipping')
                                        if k in self.options})
                raster = self.particle_raster
            elif hasattr(object, 'sample_volume'):
                raise NotImplementedError('volume rasterisation is not part of this build')
            else:
                raise ValueError(f'cannot determine raster type of object: {object}')
        if len(self.objects) >= N.T3_MAX_OBJECTS:
            raise ValueError(f'at most {N.T3_MAX_OBJECTS} objects per scene')
        if material not in self.materials:
            self.materials.append(material)
        self.objects[object] = _Obj(material, raster)

    def _raster(self):
        if self.triangle_raster is None:
            self.triangle_raster = TriangleRaster(self.engine, **self.raster_options)
        return self.triangle_raster

    def describe(self, device=None):
        """The t3_scene descriptor of the current state, with pointers on `device`
        (default: the CUDA device).  Returns (descriptor, keep-alive list)."""
        device = device or default_device()
        sc = N.t3_scene()
        keep = []
        raster = self._raster()
        # the tonemap is fused into shading unless blooming needs the HDR image
        self.engine._t3_fill_frame(sc.frame, raster.flags(self.tonemap and self.blooming is None),
                                   self.bgcolor)
        if getattr(self, 'wireframe_raster', None) is not None:
            self.wireframe_raster._t3_fill(sc.frame)
        self.lighting._t3_fill(sc.lighting)
        if hasattr(self.lighting, '_t3_fill_device'):
            self.lighting._t3_fill_device(sc.lighting, device, keep)
        base = 0
        sc.nobjects = len(self.objects)
        for o, (obj, info) in enumerate(self.objects.items()):
            ob = sc.objects[o]
            obj._t3_fill(ob.mesh, device, keep)
            if isinstance(info.raster, ParticleRaster) and not info.raster.coloring:
                ob.mesh.norms = None  # white particles (ParticleRaster(coloring=False))
            check = getattr(info.raster, 'check_faces', None)
            n = check(obj) if check else (obj.get_npars() if hasattr(obj, 'get_npars') else obj.get_nfaces())
            ob.nfaces = n
            ob.face_base = base
            base += n
            mat, uses_attr = compile_material(info.material,
                                              obj.attr_stride() if hasattr(obj, 'attr_stride') else 0,
                                              device, keep)
            if uses_attr and not ob.mesh.face_attr:
                raise ValueError('material uses FaceAttr but the mesh has no face attributes '
                                 '(mesh.set_face_attrs)')
            ob.material = mat
        return sc, keep

    def _alloc_outputs(self, dev):
        W, H = self.res
        if self.image is None or tuple(self.image.shape[:2]) != (W, H):
            self.image = torch.empty((W, H, 3), dtype=torch.float32, device=dev)
            self.face_id = torch.empty((W, H), dtype=torch.int32, device=dev)
            self.engine.depth = torch.empty((W, H), dtype=torch.int32, device=dev)
            self.depth_f = torch.empty((W, H), dtype=torch.float32, device=dev)
            self._status = torch.zeros(1, dtype=torch.int32, device=dev)

    def render(self):
        """Renders one frame into self.img (tina/scene/raster.py:168-207)."""
        require_cuda('Scene.render')
        lib = N.load()
        dev = default_device()
        if self.taa:
            self.engine.randomize_bias(self.accum.count == 0)  # raster.py:173-174
        if self._foreign_rasters():
            self._render_protocol(dev)
            self._post_process()
            return
        for obj in self.objects:
            obj.pre_compute()
        sc, keep = self.describe(dev)
        self._alloc_outputs(dev)
        mode = RASTER_MODES[self.raster_mode]
        size = C.c_size_t()
        N.check(lib.t3_workspace_size(C.byref(sc), mode, self.tile, self.bin_capacity, C.byref(size)),
                't3_workspace_size')
        if self._ws is None or self._ws.numel() < size.value:
            self._ws = N.new_workspace(size.value, dev)
        outs = N.t3_outputs()
        outs.rgb = self.image.data_ptr()
        outs.face_id = self.face_id.data_ptr()
        outs.depth = self.engine.depth.data_ptr()
        outs.depth_f = self.depth_f.data_ptr()
        for _attempt in range(3):
            N.check(lib.t3_render(C.byref(sc), mode, self.tile, self.bin_capacity,
                                  self._ws.data_ptr(), self._ws.numel(), self._status.data_ptr(),
                                  C.byref(outs), _stream()), 't3_render')
            if mode != N.T3_RASTER_BINNED or not self.check_bins:
                break
            # a bin that overflowed dropped faces: re-render with bins sized from
            # the counts this frame reached
            if not (self.status() & N.T3_STATUS_BIN_OVERFLOW):
                break
            need = C.c_int64()
            N.check(lib.t3_bin_counts_max(C.byref(sc), self.tile, self.bin_capacity,
                                          self._ws.data_ptr(), self._ws.numel(), C.byref(need),
                                          _stream()), 't3_bin_counts_max')
            self.bin_capacity = ((need.value * 5 // 4 + 32) + 31) // 32 * 32
            N.check(lib.t3_workspace_size(C.byref(sc), mode, self.tile, self.bin_capacity,
                                          C.byref(size)), 't3_workspace_size')
            if self._ws.numel() < size.value:
                self._ws = N.new_workspace(size.value, dev)
        if self.blooming is not None:
            self.blooming.apply(self.image)
            if self.tonemap:
                self._tonemap_pass.apply(self.image)
        self._post_process()
        self._keep = keep
        self._last_scene = sc

    def _post_process(self):
        if self.fxaa is not None:
            self.fxaa.apply(self.image)
        if self.taa:
            self.accum.update(self.image)

    _OWN_RASTERS = (TriangleRaster, ParticleRaster, WireframeRaster)

    def _foreign_rasters(self):
        """True when an object was added with a rasteriser of the caller's own
        (add_object(..., raster=...)): the frame then runs the three-method
        protocol object by object, as the reference's Scene.render does."""
        return any(type(info.raster) not in self._OWN_RASTERS for info in self.objects.values())

    def shader_of(self, material):
        """The Shader of `material` (Scene.shaders, tina/scene/raster.py:95-110),
        writing scene.img and, at the same pixels, the face id and float depth."""
        sh = self.shaders.get(material)
        if sh is None or sh.img is not self.image:
            sh = Shader(self.image, self.lighting, material,
                        outputs={'face_id': self.face_id, 'depth_f': self.depth_f})
            self.shaders[material] = sh
        return sh

    def _render_protocol(self, dev):
        """Scene.render's object loop (tina/scene/raster.py:176-190): clear the
        depth, then per object set_object / render_occup / render_color through
        its rasteriser, then the background of the pixels no object reached.
        The image stays HDR through the loop; the tonemap runs after it."""
        self._alloc_outputs(dev)
        self.engine.clear_depth()
        for obj, info in self.objects.items():
            shader = self.shader_of(info.material)
            info.raster.set_object(obj)
            info.raster.render_occup()
            info.raster.render_color(shader)
        bg = BackgroundShader(self.image, self.lighting, self.bgcolor,
                              outputs={'face_id': self.face_id, 'depth_f': self.depth_f})
        bg.shade_empty(self.engine)
        if self.blooming is not None:
            self.blooming.apply(self.image)
        if self.tonemap:
            self._tonemap_pass.apply(self.image)
        self._last_scene = None

    def status(self):
        """Device status bits of the last render (synchronises)."""
        lib = N.load()
        out = C.c_int32()
        N.check(lib.t3_read_status(self._status.data_ptr(), C.byref(out), _stream()), 't3_read_status')
        return out.value

    @property
    def img(self):
        """The final image (tina/scene/raster.py:209-214): float32 (W, H, 3);
        with taa, the running mean of the frames since the last clear()."""
        return self.accum.img if self.taa else self.image

    def clear(self):
        """Restarts the temporal accumulation (raster.py:230-232)."""
        if self.accum is not None:
            self.accum.clear()

    def input(self, gui):
        raise NotImplementedError('GUI camera control is not part of this headless build; '
                                  'call scene.engine.set_camera(view, proj)')
