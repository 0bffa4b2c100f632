"""Failed / FailedError, mirroring src/error/mod.rs:8-130 of smartcore."""
from __future__ import annotations

import enum


class FailedError(enum.IntEnum):
    """Error kinds (src/error/mod.rs:16-37); Display strings at :108-122."""
    FitFailed = 1
    PredictFailed = 2
    TransformFailed = 3
    FindFailed = 4
    DecompositionFailed = 5
    SolutionFailed = 6
    ParametersError = 7
    InvalidStateError = 8

    def __str__(self):
        return {
            FailedError.FitFailed: "Fit failed",
            FailedError.PredictFailed: "Predict failed",
            FailedError.TransformFailed: "Transform failed",
            FailedError.FindFailed: "Find failed",
            FailedError.DecompositionFailed: "Decomposition failed",
            FailedError.SolutionFailed: "Can't find solution",
            FailedError.ParametersError: "Error in input, check parameters",
            FailedError.InvalidStateError: "Invalid state, this should never happen",
        }[self]


class Failed(Exception):
    """Failed{err, msg}; str() is "{err}: {msg}" (src/error/mod.rs:124-128)."""

    def __init__(self, err: FailedError, msg: str):
        super().__init__(f"{err}: {msg}")
        self.err = err
        self.msg = msg

    def error(self) -> FailedError:
        return self.err

    def __eq__(self, other):
        return isinstance(other, Failed) and self.err == other.err and self.msg == other.msg

    def __hash__(self):
        return hash((int(self.err), self.msg))

    @staticmethod
    def fit(msg):
        return Failed(FailedError.FitFailed, msg)

    @staticmethod
    def predict(msg):
        return Failed(FailedError.PredictFailed, msg)

    @staticmethod
    def because(err, msg):
        return Failed(err, msg)
