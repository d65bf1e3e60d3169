"""PikeRenderer (render/pike.js:13-170) without the DOM: pass creation and tick()."""
from __future__ import annotations

import time

import numpy as np

from .passes import (AccumulatePass, CameraPass, GPUDevice, PostProcessPass, ShadeHitPass, ShadeMissPass,
                     TracePass, TraceShadowPass, read_counters)
from .scene import EnvironmentGenerator, Scene


class PikeRenderer:
    def __init__(self, scene: Scene, resolution, camera_state: dict, device: GPUDevice | None = None,
                 num_bounces: int = 4, batch_size: int | None = None, fused: bool = True):
        self.scene = scene
        self.resolution = (int(resolution[0]), int(resolution[1]))
        self.BATCH_SIZE = batch_size or self.resolution[0] * self.resolution[1]
        self.numBounces = int(num_bounces)
        self.camera = dict(camera_state)
        self.device = device
        self.fused = fused
        self.lastDraw = 0.0

    def initWebGpu(self):
        """pike.js:92-118: create every pass (the BVH and env tables are built here)."""
        if self.device is None:
            self.device = GPUDevice(0)
        d = self.device
        env = EnvironmentGenerator(self.scene.env)
        self.cameraPass = CameraPass.create(d, self.resolution, self.BATCH_SIZE)
        self.renderState = self.cameraPass.getRenderState()
        self.tracePass = TracePass.create(d, self.cameraPass, self.scene)
        self.shadePass = ShadeHitPass.create(d, self.cameraPass, self.tracePass, self.scene, env)
        self.traceShadowPass = TraceShadowPass.create(d, self.cameraPass, self.tracePass)
        self.shadeMissPass = ShadeMissPass.create(d, self.cameraPass, self.tracePass, env)
        self.accumulatePass = AccumulatePass.create(d, self.resolution, self.renderState)
        self.postProcessPass = PostProcessPass.create(d, None, None, self.accumulatePass)
        self.env = env
        return self

    def start(self):
        self.initWebGpu()
        return self

    def tick(self):
        """pike.js:120-162: one sample per pixel for every batch."""
        rs = self.renderState
        if rs.getSamples() == 0:
            self.lastDraw = time.perf_counter()
        enc = self.device.createCommandEncoder()
        rs.generateCommands(enc)
        if self.fused:
            # the whole tick in one call: every batch, misses shaded inside the traversal kernels
            self.cameraPass.setCameraState(dict(self.camera, invocationOffset=0))
            self.device.ctx.call("pk_set_camera", self.cameraPass.cameraState)
            self.device.ctx.call("pk_render_frame", self.numBounces)
            rs.incrementSamples()
            self.device.queue.submit([enc.finish()])
            return
        rs.incrementSamples()
        rs.clearColorBuffer(enc)
        n_batches = -(-self.resolution[0] * self.resolution[1] // self.BATCH_SIZE)
        for j in range(n_batches):
            rs.clearNumHitsAndMisses(enc)
            rs.clearNumRays(enc)
            self.cameraPass.setCameraState(dict(self.camera, invocationOffset=j * self.BATCH_SIZE))
            self.cameraPass.generateCommands(enc)
            for _ in range(self.numBounces):
                self.tracePass.generateCommands(enc)
                self.shadePass.generateCommands(enc)
                self.traceShadowPass.generateCommands(enc)
                self.shadeMissPass.generateCommands(enc)
        self.accumulatePass.generateCommands(enc)
        self.postProcessPass.generateCommands(enc)
        self.device.queue.submit([enc.finish()])

    def focusCamera(self) -> float:
        """pike.js:88-90: focalDepth = 1 - 1/t of the camera ray's closest hit
        (Raycaster.cast, double precision; see pk_focus_distance)."""
        import ctypes as C
        o = (C.c_double * 3)(*self.camera["pos"])
        d = (C.c_double * 3)(*self.camera["dir"])
        t, fd = C.c_double(0.0), C.c_double(0.0)
        self.device.ctx.call("pk_focus_distance", o, d, C.byref(t), C.byref(fd))
        self.camera["focalDepth"] = fd.value
        return fd.value

    def savePNG(self, path: str) -> None:
        """The tonemapped frame (PostProcessPass output) as an 8-bit PNG."""
        from .image import write_png
        write_png(path, self.image()[1][..., :3])

    def counters(self) -> dict:
        return read_counters(self.device.ctx)

    def image(self):
        return self.postProcessPass.getImage()

    def accumulation(self) -> np.ndarray:
        return self.accumulatePass.getAccumulateTexture()
