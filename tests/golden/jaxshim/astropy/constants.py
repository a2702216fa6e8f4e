from .units import Quantity, m, kg, s

G = Quantity(6.6743e-11, m ** 3 / kg / s ** 2)
