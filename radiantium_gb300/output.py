"""Film output: ResultOutput of the reference (Radiantium.Offline/ResultOutput.cs)
with its JSON keys and defaults (RendererBuilder.cs:528-543), writing the
film of a renderer as PNG (TextureUtility.SavePng: clamp(c * 255), RGBA) and
OpenEXR (TextureUtility.SaveOpenExr: linear float RGB), plus PFM.  Image row y
is film row y (neither writer flips).

Deviation: with `is_png_to_srgb` the reference's conversion loop advances
its outer index in the inner loop (ResultOutput.cs:30-36), so it converts a
few pixels of row 0 and leaves the rest black; here every pixel is
converted (the evident intent).
"""
from __future__ import annotations

import os
import struct
import zlib

import numpy as np


def _hw3(film: np.ndarray) -> np.ndarray:
    """ColorBuffer layout (x, y, rgb) -> image (y, x, rgb)."""
    return np.ascontiguousarray(np.asarray(film, dtype=np.float32).transpose(1, 0, 2))


def to_srgb(c: np.ndarray) -> np.ndarray:
    """Color3F.ToSrgb per channel (the standard sRGB transfer curve)."""
    c = np.asarray(c, dtype=np.float32)
    return np.where(c <= 0.0031308, 12.92 * c, 1.055 * np.power(np.maximum(c, 0), 1 / 2.4) - 0.055).astype(np.float32)


def save_png(film: np.ndarray, path: str, srgb: bool = False):
    img = _hw3(film)
    if srgb:
        img = to_srgb(img)
    h, w, _ = img.shape
    q = np.clip(np.rint(np.clip(img, 0.0, 1.0) * 255.0), 0, 255).astype(np.uint8)
    rgba = np.concatenate([q, np.full((h, w, 1), 255, np.uint8)], axis=2)
    raw = b"".join(b"\x00" + rgba[y].tobytes() for y in range(h))

    def chunk(tag, data):
        return struct.pack(">I", len(data)) + tag + data + struct.pack(">I", zlib.crc32(tag + data) & 0xFFFFFFFF)
    with open(path, "wb") as f:
        f.write(b"\x89PNG\r\n\x1a\n")
        f.write(chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, 8, 6, 0, 0, 0)))
        f.write(chunk(b"IDAT", zlib.compress(raw, 6)))
        f.write(chunk(b"IEND", b""))


def save_pfm(film: np.ndarray, path: str):
    img = _hw3(film)
    h, w, _ = img.shape
    with open(path, "wb") as f:
        f.write(f"PF\n{w} {h}\n-1.0\n".encode())
        f.write(np.ascontiguousarray(img[::-1]).astype("<f4").tobytes())   # PFM stores rows bottom-up


def save_exr(film: np.ndarray, path: str):
    """Single-part scanline OpenEXR, no compression, FLOAT channels B, G, R."""
    img = _hw3(film)
    h, w, _ = img.shape

    def attr(name, typ, data):
        return name.encode() + b"\x00" + typ.encode() + b"\x00" + struct.pack("<i", len(data)) + data
    chlist = b"".join(c.encode() + b"\x00" + struct.pack("<iB3xii", 2, 0, 1, 1) for c in "BGR") + b"\x00"
    box = struct.pack("<iiii", 0, 0, w - 1, h - 1)
    header = (attr("channels", "chlist", chlist) + attr("compression", "compression", b"\x00") +
              attr("dataWindow", "box2i", box) + attr("displayWindow", "box2i", box) +
              attr("lineOrder", "lineOrder", b"\x00") + attr("pixelAspectRatio", "float", struct.pack("<f", 1.0)) +
              attr("screenWindowCenter", "v2f", struct.pack("<ff", 0.0, 0.0)) +
              attr("screenWindowWidth", "float", struct.pack("<f", 1.0)) + b"\x00")
    start = 8 + len(header) + 8 * h
    line = 8 + w * 3 * 4
    offsets = struct.pack(f"<{h}Q", *[start + y * line for y in range(h)])
    body = bytearray()
    for y in range(h):
        body += struct.pack("<ii", y, w * 3 * 4)
        for c in (2, 1, 0):
            body += img[y, :, c].astype("<f4").tobytes()
    with open(path, "wb") as f:
        f.write(struct.pack("<ii", 20000630, 2) + header + offsets + bytes(body))


class ResultOutput:
    """ResultOutput (ResultOutput.cs:5-59) with the defaults of RendererBuilder.CreateOutput."""

    def __init__(self, is_save_png=False, is_png_to_srgb=False, is_save_exr=True, save_path=".", save_name="scene"):
        self.is_save_png, self.is_png_to_srgb, self.is_save_exr = is_save_png, is_png_to_srgb, is_save_exr
        self.save_path, self.save_name = save_path, save_name

    @staticmethod
    def from_config(param, search_path: str, workspace: str) -> "ResultOutput":
        if param is None:
            return ResultOutput(False, False, True, search_path, workspace)
        return ResultOutput(param.bool("is_save_png", False), param.bool("is_png_to_srgb", False),
                            param.bool("is_save_exr", True), param.str("save_path", search_path),
                            param.str("save_name", workspace))

    def save(self, renderer) -> list:
        """Writes the renderer's RenderTarget; returns the written paths."""
        film = renderer.RenderTarget
        out = []
        if self.is_save_png:
            p = os.path.abspath(os.path.join(self.save_path, f"{self.save_name}.png"))
            save_png(film, p, self.is_png_to_srgb)
            out.append(p)
        if self.is_save_exr:
            p = os.path.abspath(os.path.join(self.save_path, f"{self.save_name}.exr"))
            save_exr(film, p)
            out.append(p)
        return out
