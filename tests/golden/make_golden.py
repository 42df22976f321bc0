"""Generate golden vectors by running the reference diffrp session code.

Run from the repository root in a container where the reference tree is
present, naming its root in $DIFFRP_REFERENCE (the directory holding the
``diffrp`` package):

    DIFFRP_REFERENCE=<reference root> python tests/golden/make_golden.py [scenario ...]

The reference's own Python -- Scene / MeshObject.preprocess, the vertex
array object, the stencil-masked and full-screen interpolators, material
shading, G-buffer collection, layer composition, the flips around
nvdr_antialias -- runs on CPU tensors.  Its third-party imports that are not
installed here are replaced: ``nvdiffrast.torch`` by the oracle-backed
stand-in in ``oracle_dr.py``; trimesh.transformations and calibur by the
few standard matrix helpers the camera needs (translation, inverse, GL
perspective, focal length); the rest (loaders, path tracer, image IO) by
inert stubs that are never called.  ``device='cuda'`` allocations inside
the reference are redirected to CPU.  Output: ``tests/golden/session_*.npz``
with the inputs and the reference's outputs and gradients.  The config-1
scenario (``session_c1.npz``: 642-vertex icosphere at 512x512, L2 loss) is
stored as signatures instead of whole images to keep the file small: the
triangle-id map, a SHA-256 of the raster buffer's bytes, per-row float64
sums and a seeded sample of pixels of each image, the loss and the vertex
gradients.
"""
import importlib
import importlib.abc
import importlib.machinery
import math
import os
import sys
import types

import numpy as np

sys.dont_write_bytecode = True
HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
REF = os.environ.get("DIFFRP_REFERENCE")
sys.path.insert(0, ROOT)

import torch  # noqa: E402

STUBBED = ("trimesh", "calibur", "torch_redstone", "pyexr", "PIL", "nvdiffrast")


class _Inert(types.ModuleType):
    __path__ = []

    def __getattr__(self, name):
        if name.startswith("__"):
            raise AttributeError(name)
        m = _Inert(self.__name__ + "." + name)
        setattr(self, name, m)
        return m

    def __call__(self, *a, **k):
        raise RuntimeError("stubbed dependency %s called" % self.__name__)


class _StubFinder(importlib.abc.MetaPathFinder, importlib.abc.Loader):
    def find_spec(self, fullname, path, target=None):
        if fullname.split(".")[0] in STUBBED:
            return importlib.machinery.ModuleSpec(fullname, self, is_package=True)
        return None

    def create_module(self, spec):
        return _Inert(spec.name)

    def exec_module(self, module):
        pass


def _install_stubs():
    sys.meta_path.insert(0, _StubFinder())
    import trimesh
    import calibur
    from tests.golden import oracle_dr

    tf = types.SimpleNamespace()

    def translation_matrix(v):
        m = np.eye(4)
        m[:3, 3] = v
        return m

    tf.translation_matrix = translation_matrix
    tf.inverse_matrix = np.linalg.inv
    tf.translation_from_matrix = lambda m: np.array(m)[:3, 3].copy()
    trimesh.transformations = tf

    calibur.fov_to_focal = lambda fov, size: size / (2.0 * math.tan(fov / 2.0))

    def projection_gl_persp(w, h, cx, cy, fx, fy, near, far):
        P = np.zeros((4, 4))
        P[0, 0] = 2.0 * fx / w
        P[1, 1] = 2.0 * fy / h
        P[0, 2] = 1.0 - 2.0 * cx / w
        P[1, 2] = 2.0 * cy / h - 1.0
        P[2, 2] = -(far + near) / (far - near)
        P[2, 3] = -2.0 * far * near / (far - near)
        P[3, 2] = -1.0
        return P.astype(np.float32)

    calibur.projection_gl_persp = projection_gl_persp
    calibur.normalized = lambda x: np.asarray(x) / np.linalg.norm(x)
    import torch_redstone

    def supercat(tensors, dim=0):
        """Concatenate along ``dim``, broadcasting every other dimension."""
        nd = max(t.dim() for t in tensors)
        ts = [t.reshape((1,) * (nd - t.dim()) + tuple(t.shape)) for t in tensors]
        d = dim % nd
        shape = [max(t.shape[i] for t in ts) for i in range(nd)]
        return torch.cat([t.expand(*[t.shape[i] if i == d else shape[i] for i in range(nd)]) for t in ts], dim=d)

    torch_redstone.supercat = supercat
    import nvdiffrast
    nvdiffrast.torch = oracle_dr
    sys.modules["nvdiffrast.torch"] = oracle_dr


def _load_reference():
    if not REF:
        raise SystemExit("set DIFFRP_REFERENCE to the reference tree's root (the directory holding diffrp/)")
    if not os.path.isdir(os.path.join(REF, "diffrp")):
        raise SystemExit("reference tree not found at %s" % REF)
    sys.path.insert(0, REF)
    _install_stubs()
    for pkg in ["diffrp", "diffrp.rendering"]:
        m = types.ModuleType(pkg)
        m.__path__ = [os.path.join(REF, *pkg.split("."))]
        sys.modules[pkg] = m
    mods = {}
    for name in ["diffrp.utils.shader_ops", "diffrp.scene", "diffrp.materials", "diffrp.rendering.camera",
                 "diffrp.rendering.interpolator", "diffrp.rendering.mixin", "diffrp.rendering.surface_deferred"]:
        mods[name] = importlib.import_module(name)
    _redirect_cuda_to_cpu()
    return mods


class _TorchCPU:
    """torch with device='cuda' creation arguments redirected to CPU."""

    def __getattr__(self, name):
        attr = getattr(torch, name)
        if name in ("full", "zeros", "ones", "empty", "tensor", "arange"):
            def wrapped(*a, **k):
                if "device" in k and str(k["device"]).startswith("cuda"):
                    k["device"] = "cpu"
                return attr(*a, **k)
            return wrapped
        return attr


def _redirect_cuda_to_cpu():
    def gpu_f32(x):
        if isinstance(x, (float, int)):
            return torch.full([], x, dtype=torch.float32)
        if isinstance(x, torch.Tensor):
            return x.to(dtype=torch.float32)
        return torch.tensor(np.asarray(x), dtype=torch.float32)

    def gpu_i32(x):
        if isinstance(x, torch.Tensor):
            return x.to(dtype=torch.int32)
        return torch.tensor(np.asarray(x), dtype=torch.int32)

    for name, mod in list(sys.modules.items()):
        if name.startswith("diffrp.") and mod is not None:
            g = getattr(mod, "__dict__", {})
            if "gpu_f32" in g:
                g["gpu_f32"] = gpu_f32
            if "gpu_i32" in g:
                g["gpu_i32"] = gpu_i32
            if g.get("torch") is torch:
                g["torch"] = _TorchCPU()


# ---------------------------------------------------------------------------
# Scenarios (inputs are seeded numpy; see tests/test_gpu_session.py)
# ---------------------------------------------------------------------------
def scenario_inputs():
    from diffrp_gb300 import synthetic as S
    rng = np.random.default_rng(1234)
    sc = {}
    v, f = S.icosphere(2, 0.8)
    sc["normals"] = dict(verts=v, tris=f, h=64, w=64, fov=30.0, near=0.1, far=100.0,
                         weight=rng.normal(size=(64, 64, 3)).astype(np.float32))
    v1, f1 = S.icosphere(2, 0.5)
    c1 = rng.uniform(0, 1, (len(v1), 4)).astype(np.float32)
    v2, f2 = S.random_displaced_grid(7, seed=3, sigma=0.05)
    feat2 = rng.uniform(0, 1, (len(v2), 5)).astype(np.float32)
    th = 0.7
    M2 = np.array([[math.cos(th), 0, math.sin(th), 0.3], [0, 1, 0, 0.1], [-math.sin(th), 0, math.cos(th), 0.2],
                   [0, 0, 0, 1]], np.float32)
    M1 = np.array([[1, 0, 0, -0.45], [0, 1, 0, 0.05], [0, 0, 1, -0.2], [0, 0, 0, 1]], np.float32)
    eye = np.array([0.4, 0.9, 3.0])
    base = dict(v1=v1, f1=f1, c1=c1, M1=M1, v2=v2, f2=f2, feat2=feat2, M2=M2, h=48, w=80, fov=35.0, near=0.1,
                far=50.0, eye=eye, w_albedo=rng.normal(size=(48, 80, 4)).astype(np.float32),
                w_pos=rng.normal(size=(48, 80, 4)).astype(np.float32))
    sc["objects_masked"] = dict(base, impl="stencil_masked")
    sc["objects_full"] = dict(base, impl="full_screen")
    sc["layers"] = dict(base, impl="stencil_masked", alpha=0.6)
    # config 1 (the README example at benchmark size): icosphere with 3
    # subdivisions (642 vertices) of radius 0.8, default camera at
    # (0, 0, 3.2), fov 30, 512x512, far 100; camera-space normals through
    # nvdr_antialias; L2 loss to a seeded N(0, 0.1) target
    v, f = S.icosphere(3, 0.8)
    sc["c1"] = dict(verts=v, tris=f, h=512, w=512, fov=30.0, near=0.1, far=100.0, target_seed=0)
    return sc


def c1_target(seed, h, w):
    """N(0, 0.1) target image (h, w, 3) float32 by Box-Muller over the
    PCG64 stream's uniform doubles (stable across numpy versions, unlike
    Generator.normal's algorithm)."""
    u = np.random.default_rng(int(seed)).random((2, h, w, 3))
    z = np.sqrt(-2.0 * np.log1p(-u[0])) * np.cos(2.0 * np.pi * u[1])
    return (0.1 * z).astype(np.float32)


C1_SAMPLES = 4096


def c1_signature(out, seed=11):
    """Small signature of a config-1 render: triangle ids, SHA-256 of the
    raster bytes, per-row float64 sums and a seeded pixel sample of each
    image, the loss and the vertex gradient."""
    import hashlib
    rast = np.ascontiguousarray(out["rast"], np.float32)
    H, W = rast.shape[1:3]
    idx = np.random.default_rng(seed).choice(H * W, C1_SAMPLES, replace=False)
    sig = {"ids": rast[0, ..., 3].astype(np.int16), "rast_sha256": np.frombuffer(
        hashlib.sha256(rast.tobytes()).digest(), np.uint8), "sample_idx": idx.astype(np.int64),
        "clip": out["clip"], "loss": np.float64(out["loss"]), "grad_verts": out["grad_verts"]}
    for key in ("rast", "normals", "aa"):
        img = out[key].reshape(H, W, -1) if key != "rast" else rast[0]
        sig[key + "_rowsum"] = img.astype(np.float64).sum(axis=1)
        sig[key + "_sample"] = img.reshape(H * W, -1)[idx]
    return sig


def build_scene(api, d, name):
    """Build the scenario with a diffrp-compatible API namespace: scene,
    materials, camera modules (reference or diffrp_gb300)."""
    Scene, MeshObject = api["Scene"], api["MeshObject"]
    DefaultMaterial, SurfaceMaterial, SurfaceOutputStandard = (api["DefaultMaterial"], api["SurfaceMaterial"],
                                                               api["SurfaceOutputStandard"])
    PerspectiveCamera = api["PerspectiveCamera"]
    dev = api["device"]
    t = lambda a: torch.tensor(np.asarray(a), device=dev)  # noqa: E731
    leaves = {}
    scene = Scene()
    if name in ("normals", "c1"):
        verts = t(d["verts"]).requires_grad_(True)
        leaves["verts"] = verts
        scene.add_mesh_object(MeshObject(DefaultMaterial(), verts, t(d["tris"])))
        cam = PerspectiveCamera(fov=d["fov"], h=d["h"], w=d["w"], near=d["near"], far=d["far"])
        return scene, cam, leaves

    alpha = d.get("alpha")

    class FeatureMaterial(SurfaceMaterial):
        def shade(self, su, si):
            feat = si.custom_attrs["feat"]
            a = None if alpha is None else torch.full_like(feat[..., :1], alpha)
            return SurfaceOutputStandard(albedo=feat[..., :3], alpha=a, aovs={"feat": feat})

    v1 = t(d["v1"]).requires_grad_(True)
    c1 = t(d["c1"]).requires_grad_(True)
    v2 = t(d["v2"]).requires_grad_(True)
    feat2 = t(d["feat2"]).requires_grad_(True)
    leaves.update(v1=v1, c1=c1, v2=v2, feat2=feat2)
    scene.add_mesh_object(MeshObject(DefaultMaterial(), v1, t(d["f1"]), normals="smooth", M=t(d["M1"]), color=c1))
    scene.add_mesh_object(MeshObject(FeatureMaterial(), v2, t(d["f2"]), M=t(d["M2"]), custom_attrs={"feat": feat2}))
    cam = PerspectiveCamera(fov=d["fov"], h=d["h"], w=d["w"], near=d["near"], far=d["far"])
    pose = np.eye(4)
    pose[:3, 3] = d["eye"]
    cam.t = pose
    cam.lookat([0.0, 0.0, 0.0])
    return scene, cam, leaves


def render(api, d, name, session_cls, options_cls, ctx=None, on_session=None):
    """Render a scenario's outputs and gradients with the given session class.
    on_session(rp), when given, is called on the new session before anything
    is rendered (the tests use it to inject the reference's clip space)."""
    scene, cam, leaves = build_scene(api, d, name)
    hook = on_session if on_session is not None else (lambda rp: None)
    out = {}
    if name in ("normals", "c1"):
        rp = session_cls(scene, cam, ctx=ctx)
        hook(rp)
        n = rp.false_color_camera_space_normal()
        aa = rp.nvdr_antialias(n[..., :3])
        if name == "normals":
            (aa * torch.as_tensor(d["weight"], device=api["device"])).sum().backward()
        else:
            target = torch.as_tensor(c1_target(d["target_seed"], int(d["h"]), int(d["w"])), device=api["device"])
            loss = (aa - target).square().mean()
            loss.backward()
            out["loss"] = loss
        out.update(normals=n, aa=aa, clip=rp.clip_space(), rast=rp.rasterize()[0])
    else:
        opts = options_cls(interpolator_impl=d["impl"])
        opaque = d.get("alpha") is None
        rp = session_cls(scene, cam, opaque_only=opaque, options=opts, ctx=ctx)
        hook(rp)
        alb = rp.albedo()
        pos = rp.world_position()
        # depth() goes through transform_point4x3 (addmm), which only takes
        # (N, 3) rows: the reference supports it with the stencil-masked
        # interpolator only (full-screen buffers are (1, H, W, 3)).
        dep = rp.depth() if d["impl"] == "stencil_masked" else torch.zeros(0)
        wsn = rp.world_space_normal()
        aov = rp.aov("feat", [0.0] * 5)
        dev = api["device"]
        loss = (alb * torch.as_tensor(d["w_albedo"], device=dev)).sum() + \
            (pos * torch.as_tensor(d["w_pos"], device=dev)).sum()
        loss.backward()
        out.update(albedo=alb, world_position=pos, depth=dep, world_normal=wsn, aov=aov, clip=rp.clip_space(),
                   rast=rp.rasterize()[0], n_layers=torch.tensor(len(rp.rasterize())))
    for k, v in leaves.items():
        out["grad_" + k] = v.grad
    return {k: v.detach().cpu().numpy() for k, v in out.items()}


def edge_gradient_golden(mods, normals_out, seed=7):
    """The reference's own _EdgeGradient backward on the inputs its session
    forms for the face-soup normals scenario (surface_deferred.py:795-804)."""
    sd = mods["diffrp.rendering.surface_deferred"]
    interp = mods["diffrp.rendering.interpolator"]
    rast = torch.from_numpy(normals_out["rast"])[0]
    clip = torch.from_numpy(normals_out["clip"])
    F = clip.shape[0] // 3
    tris = torch.arange(3 * F, dtype=torch.int32).reshape(F, 3)
    frag = interp.polyfill_interpolate(clip, rast, tris[interp.float_to_triidx(rast[..., 3]) - 1], 1.0)
    frag_xy = (frag[..., :2] / frag[..., 3:4]).detach()
    flat_tris_xy = (clip[..., :2] / clip[..., 3:4])[tris.long()]
    rng = np.random.default_rng(seed)
    rgb = torch.from_numpy(np.flipud(normals_out["normals"][..., :3]).copy())
    grad = torch.from_numpy(rng.normal(size=tuple(rgb.shape)).astype(np.float32))
    leaf = frag_xy.clone().requires_grad_(True)
    rgb_leaf = rgb.clone().requires_grad_(True)
    out = sd._EdgeGradient.apply(leaf, flat_tris_xy, rast, rgb_leaf)
    out.backward(grad)
    return {"frag_xy": frag_xy.numpy(), "flat_tris_xy": flat_tris_xy.numpy(), "rast": rast.numpy(),
            "rgb": rgb.numpy(), "grad_out": grad.numpy(), "grad_frag_xy": leaf.grad.numpy(),
            "grad_rgb": rgb_leaf.grad.numpy()}


def main():
    mods = _load_reference()
    sc = mods["diffrp.scene"]
    mt = mods["diffrp.materials"]
    api = dict(Scene=sc.Scene, MeshObject=sc.MeshObject, DefaultMaterial=mt.DefaultMaterial,
               SurfaceMaterial=mt.SurfaceMaterial, SurfaceOutputStandard=mt.SurfaceOutputStandard,
               PerspectiveCamera=mods["diffrp.rendering.camera"].PerspectiveCamera, device="cpu")
    sd = mods["diffrp.rendering.surface_deferred"]
    from tests.golden import oracle_dr
    only = set(sys.argv[1:])  # scenario names to (re)generate; all when none are given
    for name, d in scenario_inputs().items():
        if only and name not in only:
            continue
        res = render(api, d, name, sd.SurfaceDeferredRenderSession, sd.SurfaceDeferredRenderSessionOptions,
                     ctx=oracle_dr.RasterizeCudaContext())
        payload = {"in_" + k: np.asarray(v) for k, v in d.items() if not isinstance(v, str)}
        if name == "c1":
            res = c1_signature(res)
        payload.update({"out_" + k: v for k, v in res.items()})
        path = os.path.join(HERE, "session_%s.npz" % name)
        np.savez_compressed(path, **payload)
        print("wrote", path, sorted(res))
        if name == "normals":
            eg = edge_gradient_golden(mods, res)
            path = os.path.join(HERE, "edge_gradient.npz")
            np.savez_compressed(path, **eg)
            print("wrote", path, sorted(eg))


if __name__ == "__main__":
    main()
