"""Host-side mirror of Pike's pass API (render/passes/*.js, render/pike.js).

The reference builds WebGPU pipelines in ``static async create(device, ...)``
factories and records one compute dispatch per ``generateCommands(encoder)``;
``PikeRenderer.tick()`` sequences them and ``device.queue.submit`` runs them.
Here the same classes, factories and method names drive libpike.so: every
``generateCommands`` enqueues the corresponding CUDA pass on the context's
stream, and ``queue.submit`` waits for it (pk_sync), raising on device-side
error flags.  Argument meaning follows the reference.
"""
from __future__ import annotations

import numpy as np

from . import _lib
from ._lib import CameraState, Context, ptr


class GPUQueue:
    def __init__(self, device: "GPUDevice"):
        self.device = device

    def submit(self, command_buffers=()):
        self.device.ctx.call("pk_sync")

    def onSubmittedWorkDone(self):
        self.device.ctx.call("pk_sync")


class CommandEncoder:
    """Passes enqueue directly on the context's stream; the encoder only marks a submission."""

    def __init__(self, device: "GPUDevice"):
        self.device = device

    def finish(self):
        return self


class GPUDevice:
    """Stands in for the WebGPU device of pike.js:92-97: one CUDA device and stream."""

    def __init__(self, cuda_device: int = 0):
        self.ctx = Context(cuda_device)
        self.queue = GPUQueue(self)

    def createCommandEncoder(self) -> CommandEncoder:
        return CommandEncoder(self)


class RenderState:
    """camera_pass.js:3-77: sample counter, env rotation and the per-frame counters."""

    def __init__(self, device: GPUDevice, resolution, batchSize: int):
        self.device = device
        self.samples = 0
        self.envTheta = 0.0
        self.resolution = tuple(int(v) for v in resolution)
        self.batchSize = int(batchSize)

    def incrementSamples(self):
        self.samples += 1

    def resetSamples(self):
        self.samples = 0

    def getSamples(self) -> int:
        return self.samples

    def setEnvRotation(self, theta: float):
        self.envTheta = float(theta)

    def generateCommands(self, commandEncoder=None):
        # clearColorBuffer + header upload {samples, envTheta, numHits=0, numMisses=0, numRays=0}
        ctx = self.device.ctx
        self.clearColorBuffer(commandEncoder)
        ctx.call("pk_set_render_state", self.samples, self.envTheta)
        ctx.call("pk_clear_hits_misses")
        ctx.call("pk_clear_rays")

    def clearNumHitsAndMisses(self, commandEncoder=None):
        self.device.ctx.call("pk_clear_hits_misses")

    def clearNumRays(self, commandEncoder=None):
        self.device.ctx.call("pk_clear_rays")

    def clearColorBuffer(self, commandEncoder=None):
        self.device.ctx.call("pk_clear_color")

    def printDebugInfo(self) -> dict:
        return read_counters(self.device.ctx)


def read_counters(ctx: Context) -> dict:
    c = np.zeros(8, np.uint32)
    ctx.call("pk_read_counters", ptr(c))
    return dict(samples=int(c[0]), num_hits=int(c[1]), num_misses=int(c[2]), num_rays=int(c[3]),
                num_shadow=int(c[4]), err=int(c[5]), rays_traced=int(c[6]) | (int(c[7]) << 32))


class CameraPass:
    """camera_pass.js:79-221 + camera.wgsl."""

    def __init__(self, device: GPUDevice, resolution, batchSize: int):
        self.device = device
        self.resolution = (int(resolution[0]), int(resolution[1]))
        self.batchSize = int(batchSize)
        self.renderState = RenderState(device, self.resolution, self.batchSize)
        self.cameraState = None

    @staticmethod
    def create(device: GPUDevice, resolution, batchSize: int) -> "CameraPass":
        inst = CameraPass(device, resolution, batchSize)
        device.ctx.call("pk_configure", inst.resolution[0], inst.resolution[1], inst.batchSize)
        return inst

    def getRenderState(self) -> RenderState:
        return self.renderState

    def setCameraState(self, state: dict):
        cs = CameraState()
        cs.pos[:] = [float(v) for v in state["pos"]]
        cs.dir[:] = [float(v) for v in state["dir"]]
        cs.fov = float(state["fov"])
        cs.focal_depth = float(state.get("focalDepth", 0.5))
        cs.aperture_size = float(state.get("apertureSize", 0.0))
        cs.distortion = float(state.get("distortion", 0.0))
        cs.bokeh = float(state.get("bokeh", 0.5))
        cs.invocation_offset = int(state.get("invocationOffset", 0))
        self.cameraState = cs

    def generateCommands(self, commandEncoder=None):
        if self.cameraState is None:
            raise _lib.PikeError(_lib.PK_ERR_STATE, "setCameraState has not been called")
        ctx = self.device.ctx
        ctx.call("pk_set_camera", self.cameraState)
        ctx.call("pk_camera")


class TracePass:
    """trace_pass.js:11-276 + trace.wgsl: builds the BVH on the GPU and traces closest hits."""

    def __init__(self, device: GPUDevice, cameraPass: CameraPass, scene):
        self.device = device
        self.cameraPass = cameraPass
        self.scene = scene

    @staticmethod
    def create(device: GPUDevice, cameraPass: CameraPass, scene) -> "TracePass":
        inst = TracePass(device, cameraPass, scene)
        scene.createBuffers(device)
        device.ctx.call("pk_bvh_build", _lib.PK_BVH_SWEEP)
        return inst

    def getBVH(self) -> dict:
        """The serialised BVH (nodes, leaf-ordered triangles, normalised vertices)."""
        ctx = self.device.ctx
        nn, nt = np.zeros(1, np.uint32), np.zeros(1, np.uint32)
        norm = np.zeros(4, np.float64)
        ctx.call("pk_bvh_info", ptr(nn), ptr(nt), ptr(norm))
        nodes = np.zeros((int(nn[0]), 5), np.int32)
        tris = np.zeros((int(nt[0]), 4), np.int32)
        verts = np.zeros((self.scene.numVertices, 4), np.float32)
        ctx.call("pk_bvh_download", ptr(nodes), ptr(tris), ptr(verts))
        return dict(nodes=nodes, tris=tris, verts=verts, center=norm[:3].copy(), scale=float(norm[3]))

    def generateCommands(self, commandEncoder=None):
        self.device.ctx.call("pk_trace")


class ShadeHitPass:
    """shade_hit_pass.js:8-181 + shade_hit.wgsl."""

    def __init__(self, device, cameraPass, tracePass, scene, envGenerator):
        self.device = device
        self.cameraPass = cameraPass
        self.tracePass = tracePass
        self.scene = scene
        self.envGenerator = envGenerator

    @staticmethod
    def create(device, cameraPass, tracePass, scene, envGenerator) -> "ShadeHitPass":
        inst = ShadeHitPass(device, cameraPass, tracePass, scene, envGenerator)
        scene.uploadMaterials(device)
        if envGenerator is not None:
            envGenerator.upload(device)
        return inst

    def generateCommands(self, commandEncoder=None):
        self.device.ctx.call("pk_shade_hit")


class TraceShadowPass:
    """trace_shadow_pass.js + trace_shadow.wgsl (any hit)."""

    def __init__(self, device, cameraPass, tracePass):
        self.device = device

    @staticmethod
    def create(device, cameraPass, tracePass) -> "TraceShadowPass":
        return TraceShadowPass(device, cameraPass, tracePass)

    def generateCommands(self, commandEncoder=None):
        self.device.ctx.call("pk_trace_shadow")


class ShadeMissPass:
    """shade_miss_pass.js + shade_miss.wgsl."""

    def __init__(self, device, cameraPass, tracePass, envGenerator):
        self.device = device

    @staticmethod
    def create(device, cameraPass, tracePass, envGenerator) -> "ShadeMissPass":
        return ShadeMissPass(device, cameraPass, tracePass, envGenerator)

    def generateCommands(self, commandEncoder=None):
        self.device.ctx.call("pk_shade_miss")


class AccumulatePass:
    """accumulate_pass.js + accumulate.wgsl (running mean)."""

    def __init__(self, device, resolution, renderState):
        self.device = device
        self.resolution = (int(resolution[0]), int(resolution[1]))
        self.renderState = renderState

    @staticmethod
    def create(device, resolution, renderState, cameraPass=None) -> "AccumulatePass":
        return AccumulatePass(device, resolution, renderState)

    def getAccumulateTexture(self) -> np.ndarray:
        w, h = self.resolution
        out = np.zeros((h, w, 4), np.float32)
        self.device.ctx.call("pk_read_accum", ptr(out))
        return out

    def generateCommands(self, commandEncoder=None):
        self.device.ctx.call("pk_accumulate")


class PostProcessPass:
    """postprocess_pass.js + postprocess.wgsl, rendering into a headless buffer
    (there is no canvas or swapchain to present to)."""

    def __init__(self, device, presentationFormat, context, accumulatePass):
        self.device = device
        self.accumulatePass = accumulatePass
        self.exposure = 1.0
        self.saturation = 1.0

    @staticmethod
    def create(device, presentationFormat=None, context=None, accumulatePass=None) -> "PostProcessPass":
        inst = PostProcessPass(device, presentationFormat, context, accumulatePass)
        inst._upload()
        return inst

    def _upload(self):
        self.device.ctx.call("pk_set_postprocess", self.exposure, self.saturation)

    def setExposure(self, exposure: float):
        self.exposure = float(exposure)
        self._upload()

    def setSaturation(self, saturation: float):
        self.saturation = float(saturation)
        self._upload()

    def generateCommands(self, commandEncoder=None):
        self.device.ctx.call("pk_postprocess")

    def getImage(self):
        w, h = self.accumulatePass.resolution
        out = np.zeros((h, w, 4), np.float32)
        out8 = np.zeros((h, w, 4), np.uint8)
        self.device.ctx.call("pk_read_display", ptr(out), ptr(out8))
        return out, out8
