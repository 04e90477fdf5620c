"""ctypes mirror of the POD types declared in include/rtp.h.

Field order and types follow the header exactly; the header in turn follows the
reference's structs (ModelParams, physics/Model.hpp:60-73; FluidKernelInputs,
physics/ocl/Fluids.hpp:17-32; BoidsRuleKernelInputs, physics/ocl/Boids.hpp:14-20;
CloudKernelInputs, physics/ocl/Clouds.hpp:15-45).
"""
import ctypes as C

# rtp_status
OK = 0
ERR_INVALID_ARGUMENT = 1
ERR_OUT_OF_MEMORY = 2
ERR_CUDA = 3
ERR_NOT_SUPPORTED = 4
ERR_STATE = 5
ERR_NO_DEVICE = 6
ERR_CAPACITY = 7

# Physics::ModelType (physics/Model.hpp:16-21)
BOIDS = 0
FLUIDS = 1
CLOUDS = 2

# Physics::Boundary (physics/Model.hpp:38-44)
BOUNCING_WALL = 0
CYCLIC_WALL = 1

# Utils::PhysicsCase (utils/Parameters.hpp:17-39)
CASE_BOIDS_SMALL = 1
CASE_BOIDS_MEDIUM = 2
CASE_BOIDS_LARGE = 3
CASE_BOIDS_XLARGE = 4
CASE_FLUIDS_DAM = 7
CASE_FLUIDS_BOMB = 8
CASE_FLUIDS_DROP = 9
CASE_CLOUDS_CUMULUS = 12
CASE_CLOUDS_HOMOGENEOUS = 13
CASE_INVALID = -1

# rtp_buffer
BUF_POS = 0
BUF_VEL = 1
BUF_PRED_POS = 2
BUF_DENSITY = 3
BUF_LAMBDA = 4
BUF_TEMP = 5
BUF_VAPOR = 6
BUF_CLOUD = 7
BUF_BUOYANCY = 8
BUF_ID = 9
BUF_CELL_ID = 10
BUF_CELL_TABLE = 11
BUF_VORTICITY = 12
BUF_ACC = 13
BUF_LAMBDA_TOTAL = 14
BUF_COLOR = 15
BUF_CAMERA_DIST = 16
BUF_DRAW_ORDER = 17
BUF_GRID_DETECTOR = 18


class ModelParams(C.Structure):
    _fields_ = [
        ("currNbParticles", C.c_uint64),
        ("maxNbParticles", C.c_uint64),
        ("boxSize", C.c_float * 3),
        ("gridRes", C.c_uint32 * 3),
        ("velocity", C.c_float),
        ("dimension", C.c_uint32),
        ("pCase", C.c_int32),
        ("maxNbPartsInCell", C.c_uint32),
    ]


class FluidParams(C.Structure):
    _fields_ = [
        ("restDensity", C.c_float),
        ("relaxCFM", C.c_float),
        ("timeStep", C.c_float),
        ("dim", C.c_uint32),
        ("isArtPressureEnabled", C.c_uint32),
        ("artPressureRadius", C.c_float),
        ("artPressureCoeff", C.c_float),
        ("artPressureExp", C.c_uint32),
        ("isVorticityConfEnabled", C.c_uint32),
        ("vorticityConfCoeff", C.c_float),
        ("xsphViscosityCoeff", C.c_float),
    ]


class BoidsParams(C.Structure):
    _fields_ = [
        ("velocityScale", C.c_float),
        ("alignmentScale", C.c_float),
        ("separationScale", C.c_float),
        ("cohesionScale", C.c_float),
    ]


class TargetParams(C.Structure):
    """rtp_target_params: the JSON "Target" group (Boids.cpp:45-51) + TargetKernelInputs."""
    _fields_ = [
        ("enabled", C.c_int32),
        ("visible", C.c_int32),
        ("radiusEffect", C.c_float),
        ("signEffect", C.c_int32),
    ]


class CloudParams(C.Structure):
    _fields_ = [
        ("dim", C.c_uint32),
        ("timeStep", C.c_float),
        ("restDensity", C.c_float),
        ("groundHeatCoeff", C.c_float),
        ("buoyancyCoeff", C.c_float),
        ("gravCoeff", C.c_float),
        ("adiabaticLapseRate", C.c_float),
        ("phaseTransitionRate", C.c_float),
        ("latentHeatCoeff", C.c_float),
        ("isTempSmoothingEnabled", C.c_uint32),
        ("relaxCFM", C.c_float),
        ("initVaporDensityCoeff", C.c_float),
        ("windCoeff", C.c_float),
    ]


class CloudEnv(C.Structure):
    _fields_ = [
        ("groundTemp0", C.c_float),
        ("lapseRate", C.c_float),
        ("heatDecay", C.c_float),
        ("windDecayX", C.c_float),
        ("windDecayZ", C.c_float),
        ("groundNx", C.c_uint32),
        ("groundNz", C.c_uint32),
    ]


class GridConstants(C.Structure):
    _fields_ = [
        ("absWall", C.c_float * 3),
        ("gridRes", C.c_uint32 * 3),
        ("cellSize", C.c_float),
        ("numCells", C.c_uint32),
        ("maxPartsInCell", C.c_uint32),
        ("effectRadius", C.c_float),
        ("effectRadiusSquared", C.c_float),
        ("poly6Coeff", C.c_float),
        ("spikyCoeff", C.c_float),
        ("maxVel", C.c_float),
        ("keyBound", C.c_uint32),
        ("keyBits", C.c_uint32),
    ]


class KernelTime(C.Structure):
    _fields_ = [
        ("name", C.c_char * 48),
        ("launches", C.c_uint64),
        ("total_ms", C.c_double),
    ]


class Metrics(C.Structure):
    _fields_ = [
        ("meanDensityError", C.c_double),
        ("maxDensityError", C.c_double),
        ("kineticEnergy", C.c_double),
        ("meanNeighbours", C.c_double),
        ("neighbourHist", C.c_uint32 * 64),
        ("meanCompression", C.c_double),
        ("pairListOverflows", C.c_uint32),
        ("pairListMax", C.c_uint32),
    ]


class BatchScene(C.Structure):
    _fields_ = [("nbParticles", C.c_uint64), ("boxSize", C.c_float * 3)]


class Tuning(C.Structure):
    _fields_ = [("lanes", C.c_uint32), ("cellFactor", C.c_float), ("tiledSweeps", C.c_uint32)]


TUNE_MAX_CANDIDATES = 32


class TuneResult(C.Structure):
    _fields_ = [
        ("best", Tuning),
        ("bestMsPerStep", C.c_double),
        ("tried", C.c_uint32),
        ("candidates", Tuning * TUNE_MAX_CANDIDATES),
        ("msPerStep", C.c_double * TUNE_MAX_CANDIDATES),
    ]


MLP_IN = 12
MLP_HIDDEN = 64
MLP_OUT = 4


class Mlp(C.Structure):
    """rtp_mlp: the warm-start network (weights row-major [out][in])."""
    _fields_ = [
        ("inMean", C.c_float * MLP_IN),
        ("inScale", C.c_float * MLP_IN),
        ("w1", (C.c_float * MLP_IN) * MLP_HIDDEN),
        ("b1", C.c_float * MLP_HIDDEN),
        ("w2", (C.c_float * MLP_HIDDEN) * MLP_HIDDEN),
        ("b2", C.c_float * MLP_HIDDEN),
        ("w3", (C.c_float * MLP_HIDDEN) * MLP_OUT),
        ("b3", C.c_float * MLP_OUT),
        ("outScale", C.c_float * MLP_OUT),
    ]


class WarmStartConfig(C.Structure):
    _fields_ = [
        ("enabled", C.c_uint32),
        ("extraIterations", C.c_uint32),
        ("guardTolerance", C.c_float),
        ("relaxAllIterations", C.c_uint32),
    ]


class SolverStats(C.Structure):
    _fields_ = [
        ("steps", C.c_uint64),
        ("reruns", C.c_uint64),
        ("sumDensityError", C.c_double),
        ("maxDensityError", C.c_double),
        ("sumFirstError", C.c_double),
    ]


class TrainConfig(C.Structure):
    _fields_ = [
        ("epochs", C.c_uint32),
        ("batch", C.c_uint32),
        ("learningRate", C.c_float),
        ("finalLrFraction", C.c_float),
        ("beta1", C.c_float),
        ("beta2", C.c_float),
        ("eps", C.c_float),
        ("weightDecay", C.c_float),
        ("lossWeights", C.c_float * MLP_OUT),
        ("seed", C.c_uint64),
    ]


MLP_ARRAYS = ("inMean", "inScale", "w1", "b1", "w2", "b2", "w3", "b3", "outScale")
MLP_TRAINABLE = ("w1", "b1", "w2", "b2", "w3", "b3")


def mlp_to_arrays(net):
    """rtp_mlp -> dict of numpy float32 arrays."""
    import numpy as np
    return {k: np.ctypeslib.as_array(getattr(net, k)).astype(np.float32).copy() for k in MLP_ARRAYS}


def mlp_from_arrays(d):
    """dict of arrays (as mlp_to_arrays) -> rtp_mlp."""
    import numpy as np
    net = Mlp()
    for k in MLP_ARRAYS:
        dst = np.ctypeslib.as_array(getattr(net, k))
        dst[...] = np.asarray(d[k], dtype=np.float32).reshape(dst.shape)
    return net


def struct_to_dict(s):
    out = {}
    for name, _ in s._fields_:
        v = getattr(s, name)
        if hasattr(v, "__len__") and not isinstance(v, (bytes, str)):
            v = list(v)
        out[name] = v
    return out


def model_params(n, max_n, box, res, dim=3, case=CASE_INVALID, velocity=1.0, cap=0):
    p = ModelParams()
    p.currNbParticles = int(n)
    p.maxNbParticles = int(max_n)
    for a in range(3):
        p.boxSize[a] = float(box[a])
        p.gridRes[a] = int(res[a])
    p.velocity = float(velocity)
    p.dimension = int(dim)
    p.pCase = int(case)
    p.maxNbPartsInCell = int(cap)
    return p
