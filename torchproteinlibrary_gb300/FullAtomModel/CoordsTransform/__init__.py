from .CoordsTransform import *
