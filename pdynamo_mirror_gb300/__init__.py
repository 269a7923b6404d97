"""pdynamo_mirror_gb300: GB300-native (sm_103a) NDDO QC/MM energy + gradient for pDynamo's QCModelMNDO path.

Public surface (mirroring pDynamo 1.9.0's names):
    QCModelMNDO, DIISSCFConverger, NBModelABFS, NBModelFull, System, ElectronicState
LangevinDynamics_SystemGeometry (Langevin dynamics of the free atoms), and, beyond the reference,
LearnedDensityGuess / LinearResponseGuess (System.DefineDensityGuess) and LangevinDynamics (many replicas at once).
The compute path is libpdg.so (CUDA, include/pdg.h); nothing here computes on the CPU.
"""

from .batch import MoleculeBatch
from .converger import DIISSCFConverger
from .dynamics import LangevinDynamics, LangevinDynamics_SystemGeometry, LangevinVelocityVerletIntegrator
from .guess import LearnedDensityGuess, LinearResponseGuess
from .mmmodel import LJParameterContainer, MMModel
from .nbmodel import NBModelABFS, NBModelFull
from .qcmodel import QCModelMNDO
from .system import ElectronicState, SCFNotConverged, System
from .trajectory import DCDTrajectoryFileReader, DCDTrajectoryFileWriter, SystemGeometryTrajectory

__all__ = ["DCDTrajectoryFileReader", "DCDTrajectoryFileWriter", "DIISSCFConverger", "LangevinDynamics", "LangevinDynamics_SystemGeometry", "LangevinVelocityVerletIntegrator", "LJParameterContainer", "MMModel", "MoleculeBatch", "SystemGeometryTrajectory", "ElectronicState", "LearnedDensityGuess", "LinearResponseGuess", "NBModelABFS", "NBModelFull", "QCModelMNDO", "SCFNotConverged", "System"]
