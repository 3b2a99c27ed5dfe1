from .Coords2RMSD import Coords2RMSD
