"""The isoparametric P2 forms (tf_setup_quaqua_p2) on the benchmark mesh, for timing and profiling:
96^3 Kuhn cubes on [-5/3,5/3]^3, P2 level set of the unit sphere, P2IF numbering; one warm-up setup, then three
timed ones (device time between stream markers; the assembly kernels' share from the library's kernel timers).

    python -m drops_gb300.profile_quaqua [n]
"""
import statistics
import sys

import drops_gb300 as tf


def main():
    n = int(sys.argv[1]) if len(sys.argv) > 1 else 96
    ctx = tf.TraceFEM()
    ctx.brick_cube(n, 5.0 / 3.0)
    ctx.levelset_analytic(tf.LS_SPHERE, [0.0, 0.0, 0.0, 1.0], True)
    na, m = ctx.distribute_dofs(tf.P2IF)
    ctx.timing(True)
    total, asm = [], []
    for rep in range(4):
        ctx.timing_reset()
        ctx.marker(6)
        newton = ctx.setup_quaqua_p2(13.0, 1e-13, 100)
        ctx.marker(7)
        if rep:
            total.append(ctx.elapsed_ms(6, 7))
            asm.append(ctx.timing_get(tf.K_ASSEMBLE)[0])
    print(f"{na} cut tets, {m} dofs: setup {statistics.median(total):.2f} ms, assembly kernels "
          f"{statistics.median(asm):.2f} ms, at most {newton} Newton iterations per point")
    ctx.close()


if __name__ == "__main__":
    main()
