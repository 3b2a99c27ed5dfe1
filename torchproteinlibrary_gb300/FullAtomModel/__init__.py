from .Angles2Coords import Angles2Coords
from .CoordsTransform import *
from .Coords2TypedCoords import *
from .PDB2Coords import *
