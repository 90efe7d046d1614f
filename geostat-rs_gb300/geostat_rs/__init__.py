"""geostat_rs -- GB300-native kriging and Vecchia likelihood (placeholder, filled below)."""
from .errors import (GeostatError, InsufficientData, DimensionMismatch, SingularSystem,
                     InvalidParameter, NoNeighbors, DuplicatePoints)
from .model import Anisotropy, Structure, VariogramModel
