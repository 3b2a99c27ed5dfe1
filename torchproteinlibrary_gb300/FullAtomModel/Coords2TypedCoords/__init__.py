from .Coords2TypedCoords import *
