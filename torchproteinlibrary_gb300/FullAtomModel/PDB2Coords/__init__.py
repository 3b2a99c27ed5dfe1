from .PDB2Coords import *
