"""Recorded canvas_ity call lists ("traces"): writer and reader.

A trace is the sequence of public ``canvas_ity::canvas`` calls an
application makes (reference API: src/canvas_ity.hpp:194-1148), serialised
in the binary layout documented in include/cy_trace.h.  The same trace is
replayed by the GB300 canvas, by the CPU oracle and by the reference, and
their pixels are compared.

`TraceWriter` mirrors the canvas API method for method; the public data
members of the C++ class (``global_composite_operation``, ``shadow_offset_x``
...) are set through ``set_<member>`` methods.
"""
from __future__ import annotations

import struct
import zlib
from dataclasses import dataclass, field
from typing import Iterator, List, Optional, Tuple

import numpy as np

MAGIC = 0x52545943
VERSION = 1

# Opcodes (include/cy_trace.h).
END, CANVAS, SCALE, ROTATE, TRANSLATE, TRANSFORM, SET_TRANSFORM = 0, 1, 2, 3, 4, 5, 6
SET_GLOBAL_ALPHA, SET_COMPOSITE_OP, SET_SHADOW_COLOR = 7, 8, 9
SET_SHADOW_OFFSET_X, SET_SHADOW_OFFSET_Y, SET_SHADOW_BLUR = 10, 11, 12
SET_LINE_WIDTH, SET_LINE_CAP, SET_LINE_JOIN, SET_MITER_LIMIT = 13, 14, 15, 16
SET_LINE_DASH_OFFSET, SET_LINE_DASH = 17, 18
SET_COLOR, SET_LINEAR_GRADIENT, SET_RADIAL_GRADIENT, ADD_COLOR_STOP, SET_PATTERN = 19, 20, 21, 22, 23
BEGIN_PATH, MOVE_TO, CLOSE_PATH, LINE_TO, QUADRATIC_CURVE_TO = 24, 25, 26, 27, 28
BEZIER_CURVE_TO, ARC_TO, ARC, RECTANGLE = 29, 30, 31, 32
FILL, STROKE, CLIP, IS_POINT_IN_PATH = 33, 34, 35, 36
CLEAR_RECTANGLE, FILL_RECTANGLE, STROKE_RECTANGLE = 37, 38, 39
SET_TEXT_ALIGN, SET_TEXT_BASELINE, SET_FONT, FILL_TEXT, STROKE_TEXT, MEASURE_TEXT = 40, 41, 42, 43, 44, 45
DRAW_IMAGE, GET_IMAGE_DATA, PUT_IMAGE_DATA, SAVE, RESTORE = 46, 47, 48, 49, 50
SET_FILL_RULE = 51                    # extension: 0 nonzero, 1 even-odd
NONZERO, EVEN_ODD = 0, 1

# Public enums (src/canvas_ity.hpp:146-156).
SOURCE_IN, SOURCE_COPY, SOURCE_OUT, DESTINATION_IN = 1, 2, 3, 4
DESTINATION_ATOP, LIGHTER, DESTINATION_OVER, DESTINATION_OUT = 7, 10, 11, 12
SOURCE_ATOP, SOURCE_OVER, EXCLUSIVE_OR = 13, 14, 15
COMPOSITE_OPS = (SOURCE_IN, SOURCE_COPY, SOURCE_OUT, DESTINATION_IN, DESTINATION_ATOP, LIGHTER,
                 DESTINATION_OVER, DESTINATION_OUT, SOURCE_ATOP, SOURCE_OVER, EXCLUSIVE_OR)
BUTT, SQUARE, CIRCLE = 0, 1, 2
MITER, BEVEL, ROUNDED = 0, 1, 2
FILL_STYLE, STROKE_STYLE = 0, 1
REPEAT, REPEAT_X, REPEAT_Y, NO_REPEAT = 0, 1, 2, 3


def _f(v: float) -> bytes:
    return struct.pack("<f", float(v))


def _i(v: int) -> bytes:
    return struct.pack("<i", int(v))


def _image_bytes(image: Optional[np.ndarray], w: int, h: int) -> bytes:
    if image is None or w <= 0 or h <= 0:
        return b""
    a = np.ascontiguousarray(image, dtype=np.uint8).reshape(-1)
    if a.size != w * h * 4:
        raise ValueError(f"image has {a.size} bytes, expected {w * h * 4}")
    return a.tobytes()


class TraceWriter:
    """Builds one canvas call list.  Method names follow the C++ API."""

    def __init__(self, width: int, height: int):
        if not (1 <= width <= 32768 and 1 <= height <= 32768):
            raise ValueError("canvas sizes must be between 1 and 32768")
        self.width, self.height = int(width), int(height)
        self._parts: List[bytes] = [struct.pack("<IIiii", MAGIC, VERSION, CANVAS, width, height)]
        self._ended = False

    def _op(self, op: int, *payload: bytes) -> "TraceWriter":
        if self._ended:
            raise RuntimeError("trace already finished")
        self._parts.append(_i(op))
        self._parts.extend(payload)
        return self

    def _ops(self, op: int, fmt: str, *vals) -> "TraceWriter":
        return self._op(op, struct.pack("<" + fmt, *vals))

    # transforms (hpp:219-294)
    def scale(self, x, y): return self._ops(SCALE, "ff", x, y)
    def rotate(self, a): return self._ops(ROTATE, "f", a)
    def translate(self, x, y): return self._ops(TRANSLATE, "ff", x, y)
    def transform(self, a, b, c, d, e, f): return self._ops(TRANSFORM, "6f", a, b, c, d, e, f)
    def set_transform(self, a, b, c, d, e, f): return self._ops(SET_TRANSFORM, "6f", a, b, c, d, e, f)
    # compositing and shadows (hpp:296-383)
    def set_global_alpha(self, a): return self._ops(SET_GLOBAL_ALPHA, "f", a)
    def set_global_composite_operation(self, op): return self._ops(SET_COMPOSITE_OP, "i", op)
    def set_shadow_color(self, r, g, b, a): return self._ops(SET_SHADOW_COLOR, "4f", r, g, b, a)
    def set_shadow_offset_x(self, v): return self._ops(SET_SHADOW_OFFSET_X, "f", v)
    def set_shadow_offset_y(self, v): return self._ops(SET_SHADOW_OFFSET_Y, "f", v)
    def set_shadow_blur(self, v): return self._ops(SET_SHADOW_BLUR, "f", v)
    # line styles (hpp:385-466)
    def set_line_width(self, v): return self._ops(SET_LINE_WIDTH, "f", v)
    def set_line_cap(self, v): return self._ops(SET_LINE_CAP, "i", v)
    def set_line_join(self, v): return self._ops(SET_LINE_JOIN, "i", v)
    def set_miter_limit(self, v): return self._ops(SET_MITER_LIMIT, "f", v)
    def set_line_dash_offset(self, v): return self._ops(SET_LINE_DASH_OFFSET, "f", v)

    def set_line_dash(self, segments: Optional[List[float]], count: Optional[int] = None):
        if count is None:
            count = 0 if segments is None else len(segments)
        payload = [_i(count), _i(0 if segments is None else 1)]
        if segments is not None and count > 0:
            payload.append(struct.pack(f"<{count}f", *segments[:count]))
        return self._op(SET_LINE_DASH, *payload)

    # fill and stroke styles (hpp:468-607)
    def set_color(self, t, r, g, b, a): return self._ops(SET_COLOR, "i4f", t, r, g, b, a)
    def set_linear_gradient(self, t, x0, y0, x1, y1):
        return self._ops(SET_LINEAR_GRADIENT, "i4f", t, x0, y0, x1, y1)
    def set_radial_gradient(self, t, x0, y0, r0, x1, y1, r1):
        return self._ops(SET_RADIAL_GRADIENT, "i6f", t, x0, y0, r0, x1, y1, r1)
    def add_color_stop(self, t, offset, r, g, b, a):
        return self._ops(ADD_COLOR_STOP, "i5f", t, offset, r, g, b, a)

    def set_pattern(self, t, image: Optional[np.ndarray], w: int, h: int, repetition: int = REPEAT):
        return self._op(SET_PATTERN, struct.pack("<5i", t, w, h, repetition, 0 if image is None else 1),
                        _image_bytes(image, w, h))

    # paths (hpp:609-848)
    def begin_path(self): return self._op(BEGIN_PATH)
    def move_to(self, x, y): return self._ops(MOVE_TO, "ff", x, y)
    def close_path(self): return self._op(CLOSE_PATH)
    def line_to(self, x, y): return self._ops(LINE_TO, "ff", x, y)
    def quadratic_curve_to(self, cx, cy, x, y): return self._ops(QUADRATIC_CURVE_TO, "4f", cx, cy, x, y)
    def bezier_curve_to(self, c1x, c1y, c2x, c2y, x, y):
        return self._ops(BEZIER_CURVE_TO, "6f", c1x, c1y, c2x, c2y, x, y)
    def arc_to(self, vx, vy, x, y, r): return self._ops(ARC_TO, "5f", vx, vy, x, y, r)
    def arc(self, x, y, r, a0, a1, ccw=False): return self._ops(ARC, "5fi", x, y, r, a0, a1, 1 if ccw else 0)
    def rectangle(self, x, y, w, h): return self._ops(RECTANGLE, "4f", x, y, w, h)
    def fill(self): return self._op(FILL)
    def stroke(self): return self._op(STROKE)
    def clip(self): return self._op(CLIP)
    def is_point_in_path(self, x, y, expected: int = -1): return self._ops(IS_POINT_IN_PATH, "ffi", x, y, expected)
    # rectangles (hpp:850-920)
    def clear_rectangle(self, x, y, w, h): return self._ops(CLEAR_RECTANGLE, "4f", x, y, w, h)
    def fill_rectangle(self, x, y, w, h): return self._ops(FILL_RECTANGLE, "4f", x, y, w, h)
    def stroke_rectangle(self, x, y, w, h): return self._ops(STROKE_RECTANGLE, "4f", x, y, w, h)
    # text (hpp:922-1026)
    def set_text_align(self, v): return self._ops(SET_TEXT_ALIGN, "i", v)
    def set_text_baseline(self, v): return self._ops(SET_TEXT_BASELINE, "i", v)

    def set_font(self, data: Optional[bytes], size: float, nbytes: Optional[int] = None):
        n = len(data) if (data is not None and nbytes is None) else (nbytes or 0)
        payload = [struct.pack("<iif", n, 0 if data is None else 1, size)]
        if data is not None and n > 0:
            payload.append(bytes(data[:n]))
        return self._op(SET_FONT, *payload)

    def _text(self, op, text: Optional[str], x, y, maxw):
        raw = b"" if text is None else text.encode("utf-8")
        return self._op(op, struct.pack("<fffii", x, y, maxw, 0 if text is None else 1, len(raw)), raw)

    def fill_text(self, text, x, y, maxw=1.0e30): return self._text(FILL_TEXT, text, x, y, maxw)
    def stroke_text(self, text, x, y, maxw=1.0e30): return self._text(STROKE_TEXT, text, x, y, maxw)

    def measure_text(self, text: Optional[str], expected: float = float("nan")):
        raw = b"" if text is None else text.encode("utf-8")
        return self._op(MEASURE_TEXT, struct.pack("<ii", 0 if text is None else 1, len(raw)), raw, _f(expected))

    # images and pixels (hpp:1028-1124)
    def draw_image(self, image: Optional[np.ndarray], w: int, h: int, x, y, to_w, to_h):
        return self._op(DRAW_IMAGE, struct.pack("<iii4f", w, h, 0 if image is None else 1, x, y, to_w, to_h),
                        _image_bytes(image, w, h))

    def get_image_data(self, w: int, h: int, x: int = 0, y: int = 0, nonnull: bool = True):
        return self._op(GET_IMAGE_DATA, struct.pack("<6i", w, h, x, y, 1 if nonnull else 0, 0))

    def put_image_data(self, image: Optional[np.ndarray], w: int, h: int, x: int, y: int):
        return self._op(PUT_IMAGE_DATA, struct.pack("<5i", w, h, x, y, 0 if image is None else 1),
                        _image_bytes(image, w, h))

    def set_fill_rule(self, rule): return self._ops(SET_FILL_RULE, "i", rule)

    def save(self): return self._op(SAVE)
    def restore(self): return self._op(RESTORE)

    def finish(self, read_back: bool = True) -> bytes:
        """End the trace; by default first read the whole canvas back."""
        if not self._ended:
            if read_back:
                self.get_image_data(self.width, self.height, 0, 0)
            self._parts.append(_i(END))
            self._ended = True
        return b"".join(self._parts)


# ---------------------------------------------------------------- reading

_FIXED = {  # opcode -> struct format of a fixed-size payload
    END: "", CANVAS: "ii", SCALE: "ff", ROTATE: "f", TRANSLATE: "ff", TRANSFORM: "6f",
    SET_TRANSFORM: "6f", SET_GLOBAL_ALPHA: "f", SET_COMPOSITE_OP: "i", SET_SHADOW_COLOR: "4f",
    SET_SHADOW_OFFSET_X: "f", SET_SHADOW_OFFSET_Y: "f", SET_SHADOW_BLUR: "f", SET_LINE_WIDTH: "f",
    SET_LINE_CAP: "i", SET_LINE_JOIN: "i", SET_MITER_LIMIT: "f", SET_LINE_DASH_OFFSET: "f",
    SET_COLOR: "i4f", SET_LINEAR_GRADIENT: "i4f", SET_RADIAL_GRADIENT: "i6f", ADD_COLOR_STOP: "i5f",
    BEGIN_PATH: "", MOVE_TO: "ff", CLOSE_PATH: "", LINE_TO: "ff", QUADRATIC_CURVE_TO: "4f",
    BEZIER_CURVE_TO: "6f", ARC_TO: "5f", ARC: "5fi", RECTANGLE: "4f", FILL: "", STROKE: "",
    CLIP: "", IS_POINT_IN_PATH: "ffi", CLEAR_RECTANGLE: "4f", FILL_RECTANGLE: "4f",
    STROKE_RECTANGLE: "4f", SET_TEXT_ALIGN: "i", SET_TEXT_BASELINE: "i", SAVE: "", RESTORE: "",
    SET_FILL_RULE: "i",
}


@dataclass
class Record:
    op: int
    args: Tuple
    data: bytes = b""          # variable payload (pixels, font, text, dash)
    expected: Optional[bytes] = None  # recorded get_image_data output
    span: Tuple[int, int] = (0, 0)    # byte range of the record in the raw call list


@dataclass
class Trace:
    width: int
    height: int
    records: List[Record] = field(default_factory=list)

    def expected_images(self) -> List[Tuple[int, int, np.ndarray]]:
        out = []
        for r in self.records:
            if r.op == GET_IMAGE_DATA and r.expected is not None:
                w, h = r.args[0], r.args[1]
                out.append((w, h, np.frombuffer(r.expected, np.uint8).reshape(h, w, 4)))
        return out

    def expected_results(self) -> List[float]:
        out = []
        for r in self.records:
            if r.op == IS_POINT_IN_PATH:
                out.append(float(r.args[2]))
            elif r.op == MEASURE_TEXT:
                out.append(float(r.args[-1]))
        return out


def _read(buf: bytes, at: int, fmt: str):
    size = struct.calcsize("<" + fmt)
    if at + size > len(buf):
        raise ValueError("truncated trace")
    return struct.unpack_from("<" + fmt, buf, at), at + size


def read_bytes(buf: bytes) -> int:
    """Bytes a replay of this call list reads back: its non-null
    get_image_data calls, compact RGBA8."""
    total = 0
    for r in parse(buf).records:
        if r.op == GET_IMAGE_DATA:
            w, h, nonnull = r.args[0], r.args[1], r.args[4]
            if nonnull and w > 0 and h > 0:
                total += w * h * 4
    return total


def parse(buf: bytes) -> Trace:
    """Parse a trace (raw, or zlib-compressed as stored in fixtures)."""
    if buf[:2] in (b"\x78\x9c", b"\x78\xda", b"\x78\x01"):
        buf = zlib.decompress(buf)
    (magic, version), at = _read(buf, 0, "II")
    if magic != MAGIC or version != VERSION:
        raise ValueError("not a canvas call list")
    trace: Optional[Trace] = None
    while True:
        start = at
        (op,), at = _read(buf, at, "i")
        if op == END:
            break
        if op in _FIXED:
            args, at = _read(buf, at, _FIXED[op])
            if op == CANVAS:
                trace = Trace(args[0], args[1])
            rec = Record(op, args)
        elif op == SET_LINE_DASH:
            (count, nonnull), at = _read(buf, at, "ii")
            vals: Tuple = ()
            if nonnull and count > 0:
                vals, at = _read(buf, at, f"{count}f")
            rec = Record(op, (count, nonnull) + tuple(vals))
        elif op in (SET_PATTERN, DRAW_IMAGE, PUT_IMAGE_DATA, GET_IMAGE_DATA):
            fmt = {SET_PATTERN: "5i", DRAW_IMAGE: "iii4f", PUT_IMAGE_DATA: "5i", GET_IMAGE_DATA: "6i"}[op]
            args, at = _read(buf, at, fmt)
            w, h = args[1:3] if op == SET_PATTERN else args[0:2]
            if op == GET_IMAGE_DATA:
                nonnull = args[5]  # has_expected
            elif op == DRAW_IMAGE:
                nonnull = args[2]
            else:
                nonnull = args[4]
            n = w * h * 4 if (nonnull and w > 0 and h > 0) else 0
            payload = buf[at:at + n]
            at += n
            rec = Record(op, args, expected=payload if op == GET_IMAGE_DATA and n else None,
                         data=b"" if op == GET_IMAGE_DATA else payload)
        elif op == SET_FONT:
            args, at = _read(buf, at, "iif")
            n = args[0] if (args[1] and args[0] > 0) else 0
            rec = Record(op, args, data=buf[at:at + n])
            at += n
        elif op in (FILL_TEXT, STROKE_TEXT):
            args, at = _read(buf, at, "fffii")
            rec = Record(op, args, data=buf[at:at + args[4]])
            at += args[4]
        elif op == MEASURE_TEXT:
            (nonnull, n), at = _read(buf, at, "ii")
            text = buf[at:at + n]
            at += n
            (exp,), at = _read(buf, at, "f")
            rec = Record(op, (nonnull, n, exp), data=text)
        else:
            raise ValueError(f"unknown opcode {op}")
        if trace is None:
            raise ValueError("trace does not start with a canvas")
        rec.span = (start, at)
        trace.records.append(rec)
    assert trace is not None
    return trace


def prefix(buf: bytes, n_records: int) -> bytes:
    """The call list cut after its first `n_records` records (the canvas
    record counts as one), ended again."""
    if buf[:2] in (b"\x78\x9c", b"\x78\xda", b"\x78\x01"):
        buf = zlib.decompress(buf)
    recs = parse(buf).records
    end = recs[min(n_records, len(recs)) - 1].span[1] if n_records > 0 else 8
    return buf[:end] + _i(END)


def canvas_size(buf: bytes) -> Tuple[int, int]:
    if buf[:2] in (b"\x78\x9c", b"\x78\xda", b"\x78\x01"):
        buf = zlib.decompress(buf)
    _, _, op, w, h = struct.unpack_from("<IIiii", buf, 0)
    if op != CANVAS:
        raise ValueError("trace does not start with a canvas")
    return w, h


def load(path) -> bytes:
    """Read a trace file, transparently decompressing zlib fixtures."""
    with open(path, "rb") as f:
        buf = f.read()
    if buf[:2] in (b"\x78\x9c", b"\x78\xda", b"\x78\x01"):
        buf = zlib.decompress(buf)
    return buf
