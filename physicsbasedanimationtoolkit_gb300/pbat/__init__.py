"""``pbat`` namespace mirroring the reference's Python module for the VBD path.

    from physicsbasedanimationtoolkit_gb300 import pbat
    data = pbat.sim.vbd.Data().with_volume_mesh(X, T).with_material(rho, mu, lam).construct()
    vbd = pbat.gpu.vbd.Integrator(data)      # or pbat.sim.vbd.Integrator(data)
    vbd.step(dt, iterations, substeps)

Both integrators run on the GPU through the C ABI of ``include/pbat_gb300.h``;
``pbat.sim.vbd.Integrator`` reproduces the reference CPU integrator's step semantics.
"""

from . import graph, gpu, sim  # noqa: F401
