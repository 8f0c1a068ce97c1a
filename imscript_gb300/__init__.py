"""GB300-native (sm_103a) simpois: Laplace, Poisson and biharmonic filling of
the NaN pixels of planar float images, behind imscript's simpois interface.

* ``imscript_gb300.simpois``  -- the solver interface (numpy or CUDA tensors)
* ``imscript_gb300.autograd`` -- torch.autograd.Function of the converged fill
* ``imscript_gb300.synth``    -- seeded synthetic workloads
* ``imscript_gb300.lib``      -- ctypes binding of libsimpois_gpu.so
"""

__all__ = ["simpois", "synth", "lib"]
