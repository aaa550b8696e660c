"""Loader for the in-tree CUDA library (``_build/libfdf_gb300.so``).

There is no CPU fallback: if the library is missing or cannot be loaded the
import raises, so a GPU run can never silently execute something else.
"""
from __future__ import annotations

import ctypes
import os

from . import build as _build

_LIB = None

c_int64_p = ctypes.POINTER(ctypes.c_int64)
c_double_p = ctypes.POINTER(ctypes.c_double)


class FdfStepInfo(ctypes.Structure):
    _fields_ = [("n_start", ctypes.c_int64), ("n_end", ctypes.c_int64), ("removed_lost", ctypes.c_int64),
                ("removed_oob", ctypes.c_int64), ("walk_evals", ctypes.c_int64), ("fp64_fallbacks", ctypes.c_int64)]


# name -> (restype, argtypes); mirrors include/fdf_gb300.h
_SIGS = {
    "fdf_ContextCreate": (ctypes.c_int, [ctypes.POINTER(ctypes.c_void_p), ctypes.c_int]),
    "fdf_ContextDestroy": (ctypes.c_int, [ctypes.c_void_p]),
    "fdf_SetGrid": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64, ctypes.c_int64, ctypes.c_void_p]),
    "fdf_SetUcat": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int]),
    "fdf_GetUcat": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int]),
    "fdf_GetGridMetrics": (ctypes.c_int, [ctypes.c_void_p] * 6),
    "fdf_SetUcont": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p]),
    "fdf_Contra2Cart": (ctypes.c_int, [ctypes.c_void_p]),
    "fdf_ResetAllParticleStatuses": (ctypes.c_int, [ctypes.c_void_p]),
    "fdf_UpdateAllParticlePositions": (ctypes.c_int, [ctypes.c_void_p]),
    "fdf_LocateAllParticlesInGrid": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p]),
    "fdf_CheckAndRemoveLostParticles": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p]),
    "fdf_CheckAndRemoveOutOfBoundsParticles": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p]),
    "fdf_InterpolateAllFieldsToSwarm": (ctypes.c_int, [ctypes.c_void_p]),
    "fdf_ScatterAllParticleFieldsToEulerFields": (ctypes.c_int, [ctypes.c_void_p]),
    "fdf_LocatePoints": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int64] + [ctypes.c_void_p] * 5),
    "fdf_InterpolatePoints": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int64] + [ctypes.c_void_p] * 3),
    "fdf_ExtractParticles": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64, ctypes.c_int64, c_int64_p]
                             + [ctypes.c_void_p] * 7),
    "fdf_AddParticles": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int64] + [ctypes.c_void_p] * 7),
    "fdf_DepositKFaceLayer": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p, ctypes.c_void_p]),
    "fdf_Contra2CartDevice": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p]),
    "fdf_SetForm": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]),
    "fdf_SetTransferRoute": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]),
    "fdf_GetTransferRoutes": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int)]),
    "fdf_SetTimeStep": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_double]),
    "fdf_SetParticleVolume": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_double]),
    "fdf_ReserveParticles": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int64]),
    "fdf_SetSwarm": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int64] + [ctypes.c_void_p] * 7),
    "fdf_SeedParticles": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int64, ctypes.c_uint64, ctypes.c_int,
                                         ctypes.c_int64, ctypes.c_double]),
    "fdf_GetSwarmSize": (ctypes.c_int, [ctypes.c_void_p, c_int64_p]),
    "fdf_GetSwarm": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int64, c_int64_p] + [ctypes.c_void_p] * 7),
    "fdf_GetScatteredFields": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]),
    "fdf_GetCornerField": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p]),
    "fdf_GetFaceDeposits": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]),
    "fdf_SetMomentumDeposit": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]),
    "fdf_GetFaceMomentum": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]),
    "fdf_PerformInitialSetup": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(FdfStepInfo)]),
    "fdf_AdvanceStep": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(FdfStepInfo)]),
    "fdf_AdvanceSteps": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]),
    "fdf_Synchronize": (ctypes.c_int, [ctypes.c_void_p]),
    "fdf_GetStream": (ctypes.c_void_p, [ctypes.c_void_p]),
    "fdf_GetLastError": (ctypes.c_char_p, [ctypes.c_void_p]),
    "fdf_GetLaunchCount": (ctypes.c_int64, [ctypes.c_void_p]),
    "fdf_SortByCell": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64, ctypes.c_void_p,
                                      ctypes.c_void_p, ctypes.c_void_p]),
    "fdf_SortByCellNoAlloc": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64, ctypes.c_void_p,
                                             ctypes.c_void_p, ctypes.c_void_p]),
    "fdf_SetProfiling": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]),
    "fdf_TestFailDeviceAllocations": (ctypes.c_int, [ctypes.c_int64]),
    "fdf_TestLocatorWaitTimeout": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64]),
    "fdf_TestLocatorTrainTimeout": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64]),
    "fdf_GetCounters": (ctypes.c_int, [ctypes.c_void_p, c_int64_p, c_int64_p, c_int64_p]),
    "fdf_GetStageTimes": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int]),
    "fdf_LocatorInit": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_uint64]),
    "fdf_LocatorTrain": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int64, ctypes.c_uint64, ctypes.c_int64,
                                        ctypes.c_int64, ctypes.c_double, ctypes.c_void_p]),
    "fdf_LocatorSetParams": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64]),
    "fdf_LocatorGetParams": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64]),
    "fdf_LocatorGetNormalization": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]),
    "fdf_LocatorGradients": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64,
                                            ctypes.c_void_p, ctypes.c_void_p]),
    "fdf_LocatorPredict": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p,
                                          ctypes.c_void_p]),
    "fdf_LocatorGetStats": (ctypes.c_int, [ctypes.c_void_p, c_int64_p, c_int64_p, c_int64_p, c_int64_p]),
    "fdf_LocatorSetMinDistance": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_double]),
    "fdf_LocatorSetInferenceType": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]),
    "fdf_ReadGridFile": (ctypes.c_int, [ctypes.c_char_p, c_int64_p, c_int64_p, c_int64_p, ctypes.c_void_p,
                                        ctypes.c_int64]),
    "fdf_WriteGridFile": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_int64, ctypes.c_int64, ctypes.c_int64,
                                         ctypes.c_void_p]),
    "fdf_WritePetscVec": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_int,
                                         ctypes.c_int]),
    "fdf_ReadPetscVec": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_void_p, ctypes.c_int64, c_int64_p, ctypes.c_int]),
    "fdf_WriteSwarmField": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_char_p, ctypes.c_char_p, ctypes.c_int]),
    "fdf_ReadSwarmField": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_char_p, ctypes.c_char_p, ctypes.c_int]),
}


def exported_symbols() -> list[str]:
    return list(_SIGS)


def load(build_if_missing: bool = True) -> ctypes.CDLL:
    """Load (building first if needed) the CUDA library; raises if it cannot."""
    global _LIB
    if _LIB is not None:
        return _LIB
    path = _build.LIB
    if not os.path.exists(path) or not _build.up_to_date():
        if not build_if_missing:
            raise RuntimeError(f"fdf_gb300 CUDA library not built: {path}")
        path = _build.build()
    lib = ctypes.CDLL(path)
    for name, (res, args) in _SIGS.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _LIB = lib
    return lib
