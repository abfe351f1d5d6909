"""Reader of the .vtu files the library and the host driver write (ASCII, or raw appended
binary with UInt32 headers): {array name: numpy array} for the points, point data and cells."""
import re

import numpy as np

_TYPES = {"Float32": np.float32, "Float64": np.float64, "Int32": np.int32, "UInt8": np.uint8}


def read_vtu(path):
    raw = open(path, "rb").read()
    head_end = raw.find(b"<AppendedData")
    head = (raw if head_end < 0 else raw[:head_end]).decode("utf-8", "replace")
    block = None
    if head_end >= 0:
        start = raw.index(b"_", head_end) + 1
        block = raw[start:]
    n = int(re.search(r"NumberOfPoints='(\d+)'", head).group(1))
    out = {}
    for m in re.finditer(r"<DataArray ([^>]*?)(/>|>(.*?)</DataArray>)", head, re.S):
        attrs = dict(re.findall(r"(\w+)='([^']*)'", m.group(1)))
        dt = _TYPES[attrs["type"]]
        comps = int(attrs.get("NumberOfComponents", "1"))
        if attrs.get("format") == "appended":
            off = int(attrs["offset"])
            nbytes = int(np.frombuffer(block[off:off + 4], dtype=np.uint32)[0])
            a = np.frombuffer(block[off + 4:off + 4 + nbytes], dtype=dt).copy()
        else:
            a = np.array(m.group(3).split(), dtype=np.float64).astype(dt)
        out[attrs["Name"]] = a.reshape(n, comps) if comps > 1 else a
    return out
