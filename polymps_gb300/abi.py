"""ctypes mirror of include/mpsgpu.h (the C ABI of libmpsgpu.so).

The structure layouts below must match the C header field for field; the CPU test
``tests/test_abi.py`` checks the sizes against the compiled library.
"""
import ctypes as C
import os

import numpy as np

_INPUT_FIELDS = [
    ("wallType", C.c_int), ("femOn", C.c_int), ("forcedOn", C.c_int),
    ("domainMin", C.c_double * 3), ("domainMax", C.c_double * 3),
    ("domainTypeBC", C.c_int), ("limitTypeBC", C.c_int),
    ("densityFluid", C.c_double), ("densityWall", C.c_double), ("KNM_VS1", C.c_double),
    ("fluidType", C.c_int),
    ("gravity", C.c_double * 3),
    ("KNM_VS2", C.c_double), ("DNS_FL1", C.c_double), ("DNS_FL2", C.c_double),
    ("dim", C.c_double), ("partDist", C.c_double), ("timeStep", C.c_double),
    ("timeSimulation", C.c_double),
    ("iterOutput", C.c_int),
    ("cflNumber", C.c_double),
    ("weightType", C.c_int), ("slipCondition", C.c_int),
    ("reS", C.c_double), ("reL", C.c_double),
    ("gradientType", C.c_int), ("gradientCorrection", C.c_int),
    ("relaxPress", C.c_double),
    ("mpsType", C.c_int),
    ("soundSpeed", C.c_double), ("gamma", C.c_double),
    ("solverType", C.c_int),
    ("alphaCompressibility", C.c_double), ("relaxPND", C.c_double),
    ("shiftingType", C.c_int),
    ("dri", C.c_double), ("coefA", C.c_double), ("machNumber", C.c_double),
    ("pndType", C.c_int),
    ("diffusiveCoef", C.c_double),
    ("repulsiveForceType", C.c_int),
    ("reRepulsiveForce", C.c_double), ("expectMaxVelocity", C.c_double),
    ("repForceCoefMitsume", C.c_double), ("repForceCoefLennardJones", C.c_double),
    ("repForceCoefMonaghanKajtar", C.c_double),
    ("EPS_RE", C.c_double),
    ("freeSurfType", C.c_int),
    ("pndThreshold", C.c_double), ("neighThreshold", C.c_double), ("npcdThreshold", C.c_double),
    ("thetaThreshold", C.c_double), ("normThreshold", C.c_double),
    ("collisionType", C.c_int),
    ("collisionRatio", C.c_double), ("distLimitRatio", C.c_double), ("lambdaCollision", C.c_double),
    ("ghost", C.c_int), ("fluid", C.c_int), ("wall", C.c_int), ("dummyWall", C.c_int),
    ("surface", C.c_int), ("inner", C.c_int), ("other", C.c_int),
]
_DERIVED_FIELDS = [
    ("epsilonZero", C.c_double),
    ("reS2", C.c_double), ("reL2", C.c_double),
    ("pndSmallZero", C.c_double), ("pndLargeZero", C.c_double), ("pndGradientZero", C.c_double),
    ("lambdaZero", C.c_double), ("numNeighZero", C.c_double),
    ("coeffViscosity", C.c_double), ("coeffViscMultiphase", C.c_double),
    ("coeffPressEMPS", C.c_double), ("coeffPressGrad", C.c_double),
    ("coeffPressWCMPS", C.c_double), ("coeffShifting1", C.c_double), ("coeffShifting2", C.c_double),
    ("coeffPPE", C.c_double), ("coeffPPESource", C.c_double),
    ("invPartDist", C.c_double), ("distCollisionLimit", C.c_double),
    ("distCollisionLimit2", C.c_double), ("restitutionCollision", C.c_double),
    ("betaPnd", C.c_double), ("betaNeigh", C.c_double), ("delta2", C.c_double),
    ("thetaArc", C.c_double), ("hThreshold2", C.c_double), ("dstThreshold2", C.c_double),
    ("normThreshold2", C.c_double),
    ("bucketSide", C.c_double), ("invBucketSide", C.c_double),
    ("numBucketsX", C.c_int), ("numBucketsY", C.c_int), ("numBucketsZ", C.c_int),
    ("numBucketsXY", C.c_int), ("numBucketsXYZ", C.c_int),
    ("derived", C.c_int),
]


class MpsParams(C.Structure):
    _fields_ = _INPUT_FIELDS + _DERIVED_FIELDS


class MpsMesh(C.Structure):
    _fields_ = [("ntri", C.c_int), ("tri_xyz", C.POINTER(C.c_double))]


class MpsStepStats(C.Structure):
    _fields_ = [
        ("numParticles", C.c_int), ("ppeIterations", C.c_int), ("ppeRefinements", C.c_int),
        ("outOfDomain", C.c_int),
        ("velMax", C.c_double), ("CFLcurrent", C.c_double),
        ("ppeRelResidual", C.c_double), ("ppeInitialRelResidual", C.c_double),
        ("ppeSolveMs", C.c_double), ("ppeAssembleMs", C.c_double), ("stepMs", C.c_double),
        ("nbrEntries", C.c_longlong), ("ppeNnz", C.c_longlong),
        ("runSteps", C.c_int), ("runPpeSolves", C.c_int),
        ("runPpeIterations", C.c_longlong), ("runPpeRefinements", C.c_longlong),
        ("ppeFallback", C.c_int), ("runPpeFallbacks", C.c_int),
    ]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


# status codes
OK, ERR_ARG, ERR_CUDA, ERR_NOMEM, ERR_UNSUPPORTED, ERR_NOT_CONVERGED, ERR_CAPACITY, \
    ERR_DOMAIN, ERR_NOGPU, ERR_SIZE_MISMATCH = range(10)

# row limit of mpsgpu_pcg_solve_static (MPSGPU_STATIC_MAX_ROWS)
STATIC_MAX_ROWS = 1 << 17

# fields (enum MpsField)
F_POS, F_VEL, F_ACC, F_ACCSTAR, F_NPCD, F_GRADC, F_CORR1, F_CORR2, F_CORR3, F_MIRROR, \
    F_WALLPOS, F_POLYNORMAL, F_FORCEWALL, F_NORMAL = range(14)
(F_PRESS, F_PRESSPPE, F_PNDI, F_PNDKI, F_PNDSKI, F_PNDSMALL, F_NPCD2, F_CONC, F_VELDIV,
 F_DIFFTERM, F_PNDWALL, F_RIW2, F_DEVDOT, F_SOURCE) = range(32, 46)
F_TYPE, F_BC, F_NUMNEIGH, F_NNEIGHWALL, F_NEARWALL = range(64, 69)
F_PRESSPPE_PREV = 46   # warm-start state (no reference array; not in SCALAR_FIELDS)
F_PRESSPPE_PREV2 = 47

VECTOR_FIELDS = set(range(14))
SCALAR_FIELDS = set(range(32, 46))
INT_FIELDS = set(range(64, 69))

FIELD_NAMES = {
    F_POS: "pos", F_VEL: "vel", F_ACC: "acc", F_ACCSTAR: "accStar", F_NPCD: "npcd",
    F_GRADC: "gradC", F_CORR1: "corr1", F_CORR2: "corr2", F_CORR3: "corr3", F_MIRROR: "mirror",
    F_WALLPOS: "wallPos", F_POLYNORMAL: "polyNormal", F_FORCEWALL: "forceWall", F_NORMAL: "normal",
    F_PRESS: "press", F_PRESSPPE: "pressPPE", F_PNDI: "pndi", F_PNDKI: "pndki",
    F_PNDSKI: "pndski", F_PNDSMALL: "pndSmall", F_NPCD2: "npcd2", F_CONC: "conc",
    F_VELDIV: "velDiv", F_DIFFTERM: "diffTerm", F_PNDWALL: "pndWall", F_RIW2: "riw2",
    F_DEVDOT: "devDot", F_SOURCE: "source",
    F_TYPE: "type", F_BC: "bc", F_NUMNEIGH: "numNeigh", F_NNEIGHWALL: "nNeighWall",
    F_NEARWALL: "nearWall",
}

# operators (enum MpsOp)
OPS = [
    "UPDATE_BUCKETS", "VISCOSITY", "ADD_GRAVITY", "PREDICT", "OUT_OF_DOMAIN", "COLLISION",
    "WALL_DISTANCE", "WALL_NPCD", "CORRECTION_MATRIX", "PND_NEIGH_NPCD", "PND_DIFFUSIVE",
    "PND_MEAN", "UPDATE_BC", "CALC_PRESS", "EXTRAPOLATE_PRESS", "PRESS_GRADIENT",
    "WALL_PRESS_GRADIENT", "WALL_VISCOSITY", "CORRECT", "SHIFTING", "DUMMY_VELOCITY",
    "INIT_PND", "PREDICT_PRESS_GRADIENT",
]
OP = {name: k for k, name in enumerate(OPS)}

SOLVER_PLAIN_FP64, SOLVER_MIXED, SOLVER_MIXED_MATFREE, SOLVER_MIXED_COMPACT = 0, 1, 2, 3
WARM_PREVIOUS, WARM_MLP, WARM_ZERO, WARM_EXTRAP, WARM_EXTRAP2 = 0, 1, 2, 3, 4
PRECISION_FP64, PRECISION_DF32 = 0, 1
MLP_NPARAM = 64 * 16 + 64 + 64 * 64 + 64 + 64 * 64 + 64 + 64 + 1
MLP_NFEAT = 16
MLP_NNORM = 2 * MLP_NFEAT + 2


def params_from_dict(d):
    """Build an MpsParams from a flat dict of its input fields (names as in the struct)."""
    p = MpsParams()
    for k, v in d.items():
        cur = getattr(p, k)
        if isinstance(cur, C.Array):
            for i, x in enumerate(v):
                cur[i] = x
        else:
            setattr(p, k, v)
    return p


def params_to_dict(p):
    out = {}
    for k, _ in MpsParams._fields_:
        v = getattr(p, k)
        out[k] = list(v) if isinstance(v, C.Array) else v
    return out


def field_spec(field, n):
    """(shape, dtype) of a field in the reference's host layout."""
    if field in VECTOR_FIELDS:
        return (n, 3), np.float64
    if field in SCALAR_FIELDS or field in (F_PRESSPPE_PREV, F_PRESSPPE_PREV2):
        return (n,), np.float64
    if field in INT_FIELDS:
        return (n,), np.int32
    raise ValueError(f"unknown field {field}")


def field_buffer(field, n):
    if field in VECTOR_FIELDS:
        return np.zeros((n, 3), dtype=np.float64)
    if field in SCALAR_FIELDS or field in (F_PRESSPPE_PREV, F_PRESSPPE_PREV2):
        return np.zeros(n, dtype=np.float64)
    if field in INT_FIELDS:
        return np.zeros(n, dtype=np.int32)
    raise ValueError(f"unknown field {field}")


def dptr(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def iptr(a):
    return a.ctypes.data_as(C.POINTER(C.c_int))


def fptr(a):
    return a.ctypes.data_as(C.POINTER(C.c_float))


def make_mesh(tri):
    """MpsMesh view of an (ntri, 9) float64 array (kept alive by the caller)."""
    if tri is None:
        return None, None
    tri = np.ascontiguousarray(tri, dtype=np.float64).reshape(-1, 9)
    m = MpsMesh(int(tri.shape[0]), dptr(tri))
    return m, tri


PKG_DIR = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG_DIR, "_build", "libmpsgpu.so")

# optional array groups of mpsgpu_write_vtu
VTU_PND, VTU_NEIGH, VTU_DEVIATION, VTU_CONCENTRATION, VTU_AUXILIAR = 1, 2, 4, 8, 16
