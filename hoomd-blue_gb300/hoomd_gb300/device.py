"""Devices (hoomd/device.py). Only the GPU device exists: the short-range MD step runs on one
GB300 with no CPU fallback."""


class Device:
    def __init__(self, notice_level=2):
        self.notice_level = notice_level

    @property
    def communicator(self):
        from hoomd_gb300.snapshot import Communicator
        return Communicator()


class GPU(Device):
    """hoomd.device.GPU: ``gpu_ids`` selects one GPU (one process drives one GPU)."""

    def __init__(self, gpu_ids=None, num_cpu_threads=None, communicator=None, msg_file=None,
                 notice_level=2):
        super().__init__(notice_level)
        if gpu_ids is not None and len(gpu_ids) > 1:
            raise ValueError("hoomd_gb300 drives exactly one GPU per process")
        self.gpu_ids = gpu_ids or [0]
        self.gpu_error_checking = True

    @property
    def devices(self):
        return [f"GPU {i}" for i in self.gpu_ids]


class CPU(Device):
    """The reference's CPU device; not provided here (no CPU path by design)."""

    def __init__(self, *args, **kwargs):
        raise NotImplementedError("hoomd_gb300 runs the MD step on the GPU only; "
                                  "use hoomd_gb300.device.GPU()")


def auto_select(*args, **kwargs):
    return GPU()
