"""One narrow-band refinement on the device, for profiling its kernels:
32^3 Kuhn cubes on [-5/3,5/3]^3 refined towards the unit sphere (width 0.05, levels 0..2, 1,062,924 tets).

    python -m drops_gb300.profile_refine [n] [width] [fine_level]
"""
import sys
import time

import drops_gb300 as tf


def main():
    n = int(sys.argv[1]) if len(sys.argv) > 1 else 32
    width = float(sys.argv[2]) if len(sys.argv) > 2 else 0.05
    fine = int(sys.argv[3]) if len(sys.argv) > 3 else 2
    ctx = tf.TraceFEM()
    ctx.brick_cube(n, 5.0 / 3.0)
    t0 = time.perf_counter()
    last, steps = ctx.mesh_refine_band(tf.LS_SPHERE, [0.0, 0.0, 0.0, 1.0], width, 0, fine)
    dt = time.perf_counter() - t0
    nv, ne, nt = ctx.mesh_info()
    print(f"refined: {nt} tets, {nv} vertices, levels 0..{last}, {steps} steps, {dt * 1e3:.1f} ms, "
          f"{ctx.launch_count()} library launches in the context")
    ctx.close()


if __name__ == "__main__":
    main()
