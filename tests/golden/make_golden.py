"""Writes the golden fixtures of this directory from the CPU oracle.

    python tests/golden/make_golden.py

The scenes are regenerated from seeds by ``pbrt_rust_gb300.generators``
(PCG32 draws and IEEE arithmetic only, so they are identical on every
machine).  The ray sets go through numpy's sin/cos, whose last bit may differ
between platforms, so they are stored beside the outputs.  Each fixture is
produced by the oracle, the C++ restatement of the reference's
BVHAccelerator / SamplerRenderer (oracle/oracle.cpp), which is itself pinned
against the reference's own known-answer tests (tests/test_kats.py).  The fixtures freeze those outputs so that

  * a change to the oracle that moves any result is caught on the CPU
    (tests/test_golden.py), and
  * the CUDA path is compared with stored values as well as with a live
    oracle run (tests/test_gpu_golden.py).

Fixtures (all small; ``.npz``, compressed):

  soup_closest.npz   4096 random triangles (C0 shape) x 4096 rays (stored,
                     (n, 8) f32): closest hits (prim, t, b1, b2 as int32
                     bit patterns) and any-hit bytes
  spheres_closest.npz  the 64-sphere scene of the 512x512 render config plus
                     its ground and light quads: 4096 incoherent rays and
                     their hits
  bvh_soup.npz       the flattened reference BVH of the 4096-triangle soup
                     (nodes, primitive order, depth)
  render_c1_48.npz   a 48x48, 2x2-jittered render of the sphere scene with
                     one point light and one area light (linear RGB f32)
  render_tris_40.npz a 40x40 render of a triangle-only scene, which every
                     implementation reproduces bit for bit
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "oracle"))

from pbrt_rust_gb300 import generators as G  # noqa: E402
from pbrt_rust_gb300.scene import SceneDescription, default_num_tasks  # noqa: E402

N_RAYS = 4096


def soup_inputs():
    prims, rays = G.ray_soup(4096, N_RAYS, seed=G.config_seed(0))
    return prims, rays


def sphere_inputs():
    prims, lights, cam, smp = G.c1_scene(res=48)
    lo, hi = np.array([-10, 0, -10], np.float32), np.array([10, 4, 10], np.float32)
    rays = G.incoherent_rays(G.PCG32(G.config_seed(1, 7)), N_RAYS, lo, hi)
    return prims, lights, cam, smp, rays


def tris_inputs():
    prims, lights, cam, smp = G.c1_scene(res=40, n_spheres=0)
    prims += G.ray_soup(300, 1, seed=11)[0]
    return prims, lights, cam, smp


def rays_array(rays: np.ndarray) -> np.ndarray:
    return np.ascontiguousarray(rays).view(np.float32).reshape(-1, 8).copy()


def as_rays(a: np.ndarray) -> np.ndarray:
    """(n, 8) f32 back to the ray record the C ABI takes."""
    from pbrt_rust_gb300 import abi
    return np.ascontiguousarray(a, dtype=np.float32).view(abi.RAY_DTYPE).reshape(-1)


def hits_array(hits: np.ndarray) -> np.ndarray:
    """(n, 4) int32: prim, then the bit patterns of t, b1, b2."""
    return np.ascontiguousarray(hits).view(np.int32).reshape(-1, 4).copy()


def main() -> int:
    import oracle as O

    prims, rays = soup_inputs()
    ob = O.OracleBVH(prims, 4, "sah")
    np.savez_compressed(HERE / "soup_closest.npz", rays=rays_array(rays), hits=hits_array(ob.intersect(rays)),
                        occluded=ob.intersect_p(rays))
    np.savez_compressed(HERE / "bvh_soup.npz", nodes=ob.nodes(), order=ob.primitive_order(),
                        depth=np.array([ob.depth()], np.uint32))

    prims, lights, cam, smp, rays = sphere_inputs()
    ob = O.OracleBVH(prims, 4, "sah")
    np.savez_compressed(HERE / "spheres_closest.npz", rays=rays_array(rays), hits=hits_array(ob.intersect(rays)),
                        occluded=ob.intersect_p(rays))
    img = O.render(SceneDescription(prims, lights, 4, "sah"), cam, smp, default_num_tasks(48, 48))
    np.savez_compressed(HERE / "render_c1_48.npz", rgb=img)

    prims, lights, cam, smp = tris_inputs()
    img = O.render(SceneDescription(prims, lights, 4, "sah"), cam, smp, default_num_tasks(40, 40))
    np.savez_compressed(HERE / "render_tris_40.npz", rgb=img)
    for p in sorted(HERE.glob("*.npz")):
        print(f"{p.name}: {p.stat().st_size} bytes")
    return 0


if __name__ == "__main__":
    sys.exit(main())
