"""A reader for the .vts files the library writes (VTK XML StructuredGrid,
inline base64 binary with UInt64 headers, little-endian Float64).  Test
infrastructure."""
import base64
import xml.etree.ElementTree as ET

import numpy as np


def read_vts(path):
    root = ET.parse(path).getroot()
    assert root.get("type") == "StructuredGrid"
    assert root.get("byte_order") == "LittleEndian" and root.get("header_type") == "UInt64"
    ext = [int(v) for v in root.find("StructuredGrid").get("WholeExtent").split()]
    dims = (ext[1] + 1, ext[3] + 1, ext[5] + 1)
    out = {}
    for da in root.iter("DataArray"):
        raw = base64.b64decode(da.text.strip())
        nbytes = int(np.frombuffer(raw[:8], dtype="<u8")[0])
        vals = np.frombuffer(raw[8:8 + nbytes], dtype="<f8")
        ncomp = int(da.get("NumberOfComponents"))
        out[da.get("Name")] = vals.reshape(-1, ncomp) if ncomp > 1 else vals
    return dims, out
