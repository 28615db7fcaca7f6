"""``jax.sharding`` stand-ins for the single-device NumPy shim."""


class PartitionSpec(tuple):
    def __new__(cls, *parts):
        return super().__new__(cls, parts)


class NamedSharding:
    def __init__(self, mesh, spec):
        self.mesh = mesh
        self.spec = spec


class AxisType:
    Auto = "auto"
    Explicit = "explicit"
    Manual = "manual"
