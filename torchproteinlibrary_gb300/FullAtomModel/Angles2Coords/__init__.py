from .Angles2Coords import Angles2Coords, Angles2CoordsFunction, convertStringList, convertString
