"""taichi_three_gb300 -- Tina's triangle rasteriser and deferred shading pass,
rebuilt for one GB300 (sm_103a) GPU.

Drop-in names follow Tina (taichi-dev/taichi_three): `import taichi_three_gb300
as tina`, then tina.Scene, tina.SimpleMesh, tina.PBR, ... as in the reference's
docs.  Rendering runs in hand-written CUDA kernels behind the C ABI of
include/tina3.h; there is no CPU fallback.
"""
__version__ = (0, 1, 1)

from .matrix import (affine, eularXYZ, frustum, identity, lookat, orbit_camera, ortho,
                     orthogonal, perspective, quaternion, scale, translate)
from .nodes import ChessboardTexture, Const, FaceAttr, Input, Node, Param, Texture
from .materials import (AddMaterial, Classic, CookTorrance, Diffuse, Emission, FresnelFactor,
                        IMaterial, Lambert, Lamp, MixMaterial, PBR, Phong, ScaleMaterial,
                        compile_material)
from .lighting import Lighting
from .mesh import (MAX, ConnectiveMesh, MeshFlatNormal, MeshFlipCulling, MeshFlipNormal, MeshGrid,
                   MeshModel, MeshNoCulling, MeshSmoothNormal, MeshToWire, MeshTransform, PrimitiveMesh, SimpleMesh,
                   SimpleParticles)
from .engine import Engine
from .scene import BackgroundShader, ParticleRaster, Scene, Shader, TriangleRaster, WireframeRaster
from .postp import Accumator, Blooming, FXAA, ToneMapping, aces_tonemap
from .skybox import IBLTables, PlainSkybox, Skybox, SkyboxLighting, procedural_sky
from .pipeline import FramePipeline
from . import workloads
from .assimp import readobj
from .mlp import IBLNet, train_for_skybox
from . import colour
from .batch import BatchRenderer
from .autotune import Autotuner, tune_scene
from .animate import FrameGraph
