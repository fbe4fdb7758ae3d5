"""The bounds-check build (-DPLT_BOUNDS_CHECK=1, plt_bounds.cuh): every checked index of the BSDF
batch (sort permutation) and of the render pass (queue entries, path ids, bounce records, triangles,
materials, deferred walk and replay tasks, the image accumulator) is compared with its buffer's
bound, and a violation is reported through plt_check_status (PLT_BOUNDS_VIOLATION) with its site,
index and bound instead of being made.  This test builds that variant of the library into its own
directory and runs, in a child process that loads it, a mixed-material batch, closest-hit and any-hit
traversal, a render with manifold walks and deferred replays over several frames, and a three-scene
batched render (HWSS 8, learned proposal): every call must report no violation.
"""
import os
import subprocess
import sys

import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CHILD = r'''
import sys
import numpy as np
import torch
sys.path.insert(0, sys.argv[2])
from pltfalcor_gb300 import capi, scene as S, spectra, workloads as W
capi.load_library(sys.argv[1])
from pltfalcor_gb300.bsdf import DeviceBatch, PLTContext

def ok(ctx, what):
    st = ctx.check_status()
    assert st == capi.PLT_OK, "%s: %s %s" % (what, capi.STATUS_NAMES.get(st, st), ctx.last_bounds_violation())

prof, _ = spectra.standard_profiles()
wl = W.mixed_material_batch(n=3 * 8192 + 776, profiles=prof)   # a partial last tile
ctx = PLTContext()
ctx.set_spectral_profiles(prof)
ctx.set_materials(wl.records)
b = DeviceBatch(wl)
ops = capi.OP_EVAL | capi.OP_SAMPLE | capi.OP_PDF | capi.OP_LAMBDA_PDF
ctx.batch(b.queries(), b.results(ops), ops)
ok(ctx, "bsdf batch")

sc = S.procedural_scene(n_spheres=20, sphere_level=2, n_quads=50, box_subdiv=8)
ctx.set_scene(sc.vertices, sc.indices, sc.tri_material)
o, d = S.random_rays(20000, 5, sc.bounds, sc.triangle_vertices())
n = len(o) // 3
go, gd = torch.from_numpy(o).cuda(), torch.from_numpy(d).cuda()
prim = torch.zeros(n, dtype=torch.int32, device="cuda")
occ = torch.zeros(n, dtype=torch.int32, device="cuda")
ctx.trace_closest(ctx.rays(go, gd), prim)
ctx.trace_any(ctx.rays(go, gd), occ)
ok(ctx, "trace")
ctx.close()

room = S.small_scene()
ctx = PLTContext({"max_bounces": 8, "hwss": 4, "do_mnee": 1})
ctx.load_scene(room, prof)
w, h = 96, 64
out = torch.zeros((h, w, 4), dtype=torch.float32, device="cuda")
ctx.render(S.room_camera(w, h), w, h, out, 0, 3)
torch.cuda.synchronize()
ok(ctx, "render")
assert np.isfinite(out.cpu().numpy()).all()
ctx.close()

rooms = [S.procedural_scene(seed=11, n_spheres=6, sphere_level=2, n_quads=30, box_subdiv=4),
         S.procedural_scene(seed=12, n_spheres=2, sphere_level=3, n_quads=10, box_subdiv=6),
         S.procedural_scene(seed=13, n_spheres=10, sphere_level=1, n_quads=50, box_subdiv=3)]
ctx = PLTContext({"max_bounces": 6, "hwss": 8, "do_mnee": 1, "learned_proposal": 1, "learned_proposal_prob": 0.25})
recs, offs = S.merged_materials(rooms)
ctx.set_spectral_profiles(prof)
ctx.set_materials(recs)
ids = [ctx.add_scene(r, off) for r, off in zip(rooms, offs)]
ctx.proposal_init(3)
ctx.proposal_train(8, batch=8192, lr=1e-3, seed=1)
sizes = [(48, 32), (40, 40), (64, 24)]
outs = [torch.zeros((hh, ww, 4), dtype=torch.float32, device="cuda") for ww, hh in sizes]
views = [(i, S.room_camera(ww, hh), ww, hh, t) for i, (ww, hh), t in zip(ids, sizes, outs)]
ctx.render_scenes(views, 0, 2)
torch.cuda.synchronize()
ok(ctx, "scene set")
ctx.close()
print("no bounds violation")
'''


def test_bounds_check_build_reports_no_violation():
    pytest.importorskip("torch")
    from pltfalcor_gb300 import build
    lib = build.build(defines=["PLT_BOUNDS_CHECK=1"], build_dir=os.path.join(ROOT, "pltfalcor_gb300", "_build_bounds"))
    r = subprocess.run([sys.executable, "-c", CHILD, lib, ROOT], capture_output=True, text=True, timeout=1200)
    assert r.returncode == 0, r.stdout[-3000:] + r.stderr[-3000:]
    assert "no bounds violation" in r.stdout
