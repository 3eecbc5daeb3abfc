"""The ctypes mirror of include/pyre_cuda.h has the C structs' layout: a C
program compiled against the header prints every struct's size and every
field's offset, and each must equal the ctypes class's."""
import ctypes as C
import shutil
import subprocess
from pathlib import Path

import pytest

from pyre_gb300 import native as N

ROOT = Path(__file__).resolve().parents[1]

PAIRS = {
    "pyre_bvh2_node": N.Bvh2Node,
    "pyre_mesh_desc": N.MeshDesc,
    "pyre_instance_desc": N.InstanceDesc,
    "pyre_material_desc": N.MaterialDesc,
    "pyre_quad_light_desc": N.QuadLightDesc,
    "pyre_env_desc": N.EnvDesc,
    "pyre_scene_desc": N.SceneDesc,
    "pyre_scene_info": N.SceneInfo,
    "pyre_rays": N.Rays,
    "pyre_hits": N.Hits,
    "pyre_camera_desc": N.CameraDesc,
    "pyre_render_params": N.RenderParams,
    "pyre_film": N.Film,
    "pyre_render_stats": N.RenderStats,
    "pyre_gradients": N.Gradients,
    "pyre_batch_job": N.BatchJob,
}


def test_ctypes_structs_match_the_header(tmp_path):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    lines = ["#include <stddef.h>", "#include <stdio.h>", '#include "pyre_cuda.h"', "int main(void) {"]
    for cname, cls in PAIRS.items():
        lines.append(f'    printf("{cname} size %zu\\n", sizeof({cname}));')
        for field, _ in cls._fields_:
            lines.append(f'    printf("{cname} {field} %zu\\n", offsetof({cname}, {field}));')
    lines += ["    return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    r = subprocess.run([cc, "-std=c11", "-I", str(ROOT / "include"), str(src), "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split("\n")
    c_layout = {}
    for line in out:
        if line:
            cname, what, value = line.split()
            c_layout[(cname, what)] = int(value)
    for cname, cls in PAIRS.items():
        assert C.sizeof(cls) == c_layout[(cname, "size")], cname
        for field, _ in cls._fields_:
            assert getattr(cls, field).offset == c_layout[(cname, field)], (cname, field)


def test_python_constants_match_the_header():
    """Every PYRE_* value the header defines and native.py mirrors is equal."""
    import re
    text = (ROOT / "include" / "pyre_cuda.h").read_text()
    defines = {m.group(1): int(m.group(2)) for m in
               re.finditer(r"^#define (PYRE_[A-Z0-9_]+) (-?\d+)\b", text, re.M)}
    mirrored = {name: getattr(N, name) for name in defines if hasattr(N, name)}
    assert len(mirrored) >= 15
    for name, value in mirrored.items():
        assert value == defines[name], name


def _c_struct_fields(header: str) -> dict:
    import re
    out = {}
    for m in re.finditer(r"typedef struct (pyre_\w+) \{(.*?)\} \1;", header, re.S):
        body = re.sub(r"/\*.*?\*/", "", m.group(2), flags=re.S)
        fields = []
        for decl in body.split(";"):
            decl = re.sub(r"\[[^\]]*\]", "", decl.strip())
            if not decl:
                continue
            parts = decl.split(",")
            fields.append(parts[0].split()[-1].lstrip("*"))
            fields += [q.strip().lstrip("*") for q in parts[1:]]
        out[m.group(1)] = fields
    return out


def test_rust_binding_sketch_matches_the_header():
    """The #[repr(C)] structs of the Rust binding (include/pyre_cuda_ffi.rs)
    list the C structs' fields in the same order (no Rust compiler checks them
    here)."""
    import re
    doc = (ROOT / "include" / "pyre_cuda_ffi.rs").read_text()
    cs = _c_struct_fields((ROOT / "include" / "pyre_cuda.h").read_text())
    rust = {m.group(1): re.findall(r"pub (\w+):", m.group(2))
            for m in re.finditer(r"#\[repr\(C\)\] pub struct (\w+) \{(.*?)\}", doc, re.S)}
    assert len(rust) >= 16
    for name, fields in rust.items():
        cname = "pyre_" + re.sub(r"(?<!^)(?=[A-Z])", "_", name[len("Pyre"):]).lower()
        assert cs.get(cname) == fields, (name, fields, cs.get(cname))
