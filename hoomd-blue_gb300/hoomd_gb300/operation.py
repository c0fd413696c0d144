"""hoomd.operation.AutotunedObject (hoomd/operation.py:391-497): kernel parameters of the GPU
kernels an object launches, and the search for the fastest of them.

The search is the engine's (``IntegratorTwoStep.autotune``): at the next run every candidate
launch configuration is timed on the live state, which is restored afterwards, and the fastest is
kept. Unlike the reference, whose tuner varies the parameters over the first thousands of steps
by default, the search runs only after `tune_kernel_parameters`: a tuned configuration changes
summation orders, so the defaults keep a run reproducible bit for bit."""

from hoomd_gb300.error import DataAccessError


class AutotunedObject:
    """An object whose ``_cpp_obj`` launches tunable kernels."""

    @property
    def kernel_parameters(self):
        """dict[str, tuple[int]]: kernel name -> launch parameters in use ("pair": (block size,
        threads per particle); "nlist": (block size, threads per particle), where 32 threads per
        particle is the candidate-stream build and 1 the lane-per-particle build)."""
        if getattr(self, "_cpp_obj", None) is None:
            raise DataAccessError("kernel_parameters")
        return self._cpp_obj.getAutotunerParameters()

    @kernel_parameters.setter
    def kernel_parameters(self, parameters):
        if getattr(self, "_cpp_obj", None) is None:
            raise DataAccessError("kernel_parameters")
        self._cpp_obj.setAutotunerParameters({k: tuple(v) for k, v in dict(parameters).items()})
        sim = getattr(self, "_simulation", None)
        if sim is not None:
            sim._state_changed()  # the captured steps hold the launch configuration

    @property
    def is_tuning_complete(self):
        """bool: True unless a search was requested and has not run yet."""
        if getattr(self, "_cpp_obj", None) is None:
            raise DataAccessError("is_tuning_complete")
        return bool(self._cpp_obj.isAutotuningComplete())

    def tune_kernel_parameters(self):
        """Search the kernel parameters at the start of the next run."""
        if getattr(self, "_cpp_obj", None) is None:
            raise RuntimeError("Call Simulation.run() before tune_kernel_parameters.")
        self._cpp_obj.startAutotuning()
