"""Host-side mirror of naeioi/PBF-CUDA's ``SSFRenderer`` (fluids/SSFRenderer.h:4-74).

The screen-space fluid surface of the particles, rendered by the CUDA kernels
of libpbf.so (include/pbf_ssf.h) into headless device images instead of an
OpenGL framebuffer: ``render(pos)`` runs the reference's depth splat,
thickness splat, smoothing passes, normal restoration and shading
(fluids/SSFRenderer.cpp:113-146) and returns the colour image as a CUDA
tensor (H, W, 4), row 0 at the bottom as in OpenGL.

The reference's world is z-up (its camera's up is +z, fluids/Camera.cpp:66,
and trace_color's floor is the plane z = 0, fluids/shader/SSFshading.f.glsl:50-72);
``z_up()`` turns the y-up particle states of this package's scenes into it.
"""
from __future__ import annotations

import ctypes
from pathlib import Path
from typing import Optional, Sequence

import numpy as np
import torch

from ._abi import PbfSsfParams, PbfSsfProfile, check, lib
from .simulator import _stream_handle, _vec3

SHADING = {"full": 0, "depth": 1, "thick": 2, "normal": 3, "fresnel": 4, "reflect": 5, "refract": 6,
           "refract_tinted": 7}


def ssf_default_params(width: Optional[int] = None, height: Optional[int] = None) -> PbfSsfParams:
    """The reference's renderer settings and camera (pbf_ssf_params_default),
    optionally at another image size (the camera's aspect follows it)."""
    p = PbfSsfParams()
    lib().pbf_ssf_params_default(ctypes.byref(p))
    if width is not None or height is not None:
        p.width = int(width or p.width)
        p.height = int(height or p.height)
        look_at(p, (1.0, -5.0, 2.0), (0.0, 0.0, 1.5))
    return p


def look_at(p: PbfSsfParams, pos: Sequence[float], focus: Sequence[float], fov_deg: float = 60.0) -> PbfSsfParams:
    """Camera(pos, focus, aspect) (fluids/Camera.cpp:64-96): fills p's matrices."""
    check(lib().pbf_ssf_look_at(ctypes.byref(p), _vec3(pos), _vec3(focus), float(fov_deg)), "pbf_ssf_look_at")
    return p


def z_up(pos: torch.Tensor) -> torch.Tensor:
    """(x, y, z) -> (x, -z, y): a y-up state in the reference's z-up world."""
    out = torch.empty_like(pos)
    out[:, 0] = pos[:, 0]
    out[:, 1] = -pos[:, 2]
    out[:, 2] = pos[:, 1]
    out[:, 3] = pos[:, 3]
    return out


class SSFRenderer:
    """One renderer instance with its device images (W x H)."""

    def __init__(self, params: Optional[PbfSsfParams] = None):
        self._L = lib()
        self.params = (params or ssf_default_params()).copy()
        self._h = ctypes.c_void_p()
        check(self._L.pbf_ssf_create(ctypes.byref(self.params), ctypes.byref(self._h)), "pbf_ssf_create")

    @property
    def width(self) -> int:
        return self.params.width

    @property
    def height(self) -> int:
        return self.params.height

    def close(self) -> None:
        if self._h:
            self._L.pbf_ssf_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def load_params(self, params: PbfSsfParams) -> None:
        """loadParams (fluids/SSFRenderer.cpp:280-288): settings for the next render."""
        check(self._L.pbf_ssf_set_params(self._h, ctypes.byref(params)), "pbf_ssf_set_params")
        self.params = params.copy()

    def set_sky(self, faces: Optional[np.ndarray]) -> None:
        """Cube map (6, S, S, 3) float32 in GL face order, or None for the uniform sky colour."""
        if faces is None:
            check(self._L.pbf_ssf_set_sky(self._h, None, 0), "pbf_ssf_set_sky")
            return
        f = np.ascontiguousarray(faces, dtype=np.float32)
        if f.ndim != 4 or f.shape[0] != 6 or f.shape[1] != f.shape[2] or f.shape[3] != 3:
            raise ValueError("sky faces must be (6, S, S, 3)")
        check(self._L.pbf_ssf_set_sky(self._h, f.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), f.shape[1]),
              "pbf_ssf_set_sky")

    def render(self, pos: torch.Tensor, n: Optional[int] = None, color: Optional[torch.Tensor] = None,
               stream=None) -> torch.Tensor:
        """SSFRenderer::render(p_vao, nparticle): the first n rows of pos
        ((>= n, 4) float32 on the GPU).  color: (H, W, 4) float32 image to draw
        into (pixels without fluid keep their value); a zeroed one by default."""
        n = pos.shape[0] if n is None else int(n)
        if not (pos.is_cuda and pos.dtype == torch.float32 and pos.dim() == 2 and pos.shape[1] == 4
                and pos.shape[0] >= n and pos.is_contiguous()):
            raise ValueError("pos must be a contiguous CUDA float32 tensor of shape (>= n, 4)")
        if color is None:
            color = torch.zeros((self.height, self.width, 4), dtype=torch.float32, device=pos.device)
        elif not (color.is_cuda and color.dtype == torch.float32 and tuple(color.shape) == (self.height, self.width, 4)
                  and color.is_contiguous()):
            raise ValueError(f"color must be a contiguous CUDA float32 tensor of shape ({self.height}, {self.width}, 4)")
        check(self._L.pbf_ssf_render(self._h, pos.data_ptr() if n else None, n, color.data_ptr(),
                                     _stream_handle(stream)), "pbf_ssf_render")
        return color

    def images(self, device=None, stream=None) -> dict:
        """The last render's smoothed depth (H, W), thickness (H, W) and normal_D (H, W, 4)."""
        dev = device or torch.device("cuda", torch.cuda.current_device())
        out = {"depth": torch.empty((self.height, self.width), dtype=torch.float32, device=dev),
               "thick": torch.empty((self.height, self.width), dtype=torch.float32, device=dev),
               "normal_D": torch.empty((self.height, self.width, 4), dtype=torch.float32, device=dev)}
        check(self._L.pbf_ssf_images(self._h, out["depth"].data_ptr(), out["thick"].data_ptr(),
                                     out["normal_D"].data_ptr(), _stream_handle(stream)), "pbf_ssf_images")
        return out

    def profile_enable(self, on: bool = True) -> None:
        check(self._L.pbf_ssf_profile_enable(self._h, int(bool(on))), "pbf_ssf_profile_enable")

    def profile(self) -> dict:
        prof = PbfSsfProfile()
        check(self._L.pbf_ssf_profile_read(self._h, ctypes.byref(prof)), "pbf_ssf_profile_read")
        return prof.as_dict()


def write_ppm(path, color, background=(0.0, 0.0, 0.0)) -> Path:
    """An (H, W, 4) colour image (row 0 at the bottom) as a binary PPM, top row
    first; alpha 0 pixels take the background colour."""
    c = color.detach().cpu().numpy() if isinstance(color, torch.Tensor) else np.asarray(color)
    rgb = np.where(c[..., 3:4] > 0, c[..., :3], np.asarray(background, np.float32))
    img = (np.clip(rgb[::-1], 0.0, 1.0) * 255.0 + 0.5).astype(np.uint8)
    path = Path(path)
    with open(path, "wb") as f:
        f.write(f"P6 {img.shape[1]} {img.shape[0]} 255\n".encode())
        f.write(img.tobytes())
    return path
