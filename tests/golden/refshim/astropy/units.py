import math

deg = math.pi / 180
mm = 1.0
