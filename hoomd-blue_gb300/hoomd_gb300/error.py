"""hoomd.error: the exception types of the reference's Python API (hoomd/error.py)."""


class DataAccessError(RuntimeError):
    """Data available only while the object is attached to a simulation that has run."""

    def __init__(self, data_name):
        self.data_name = data_name
        super().__init__(f"The property {data_name} is unavailable until the simulation runs.")
