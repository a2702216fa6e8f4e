"""Units as (SI scale, dimension exponents) with *, / and ** and Quantity.to."""


class Unit:
    def __init__(self, scale, dims):
        self.scale = float(scale)
        self.dims = dict(dims)

    def _combine(self, other, sign):
        d = dict(self.dims)
        for k, v in other.dims.items():
            d[k] = d.get(k, 0) + sign * v
        return Unit(self.scale * other.scale ** sign, {k: v for k, v in d.items() if v != 0})

    def __mul__(self, o):
        if isinstance(o, Unit):
            return self._combine(o, 1)
        return Quantity(o, self)

    __rmul__ = __mul__

    def __truediv__(self, o):
        return self._combine(o, -1)

    def __pow__(self, p):
        return Unit(self.scale ** p, {k: v * p for k, v in self.dims.items()})


class Quantity:
    def __init__(self, value, unit):
        self.value = value
        self.unit = unit

    def __truediv__(self, o):
        if isinstance(o, Unit):
            return Quantity(self.value, self.unit / o)
        return Quantity(self.value / o, self.unit)

    def __mul__(self, o):
        if isinstance(o, Unit):
            return Quantity(self.value, self.unit * o)
        return Quantity(self.value * o, self.unit)

    def to(self, unit):
        if self.unit.dims != unit.dims:
            raise ValueError("incompatible units")
        return Quantity(self.value * self.unit.scale / unit.scale, unit)


m = Unit(1.0, {"m": 1})
km = Unit(1e3, {"m": 1})
s = Unit(1.0, {"s": 1})
kg = Unit(1.0, {"kg": 1})
kpc = Unit(3.0856775814913673e19, {"m": 1})
Msun = Unit(1.988409870698051e30, {"kg": 1})
Gyr = Unit(3.15576e16, {"s": 1})
