"""SimParams as a ctypes structure, byte-identical to include/sph_params.h.

The C layout is the reference's ``struct SimParams`` (source/CUDA/Params.cuh:
53-114); the offsets are asserted below and again in C by static_asserts.
"""
from __future__ import annotations

import ctypes

# BndType / BndEff / ClrType / AccType (Params.cuh:24-41)
BND_BOX, BND_CYL_Y, BND_CYL_Z, BND_CYL_YZ, BND_SPHERE, BND_PUMP_Y = range(6)
BND_EFF_NONE, BND_EFF_WRAP, BND_EFF_CYCLE, BND_EFF_WAVE = range(4)
CLR_DENS, CLR_ACCEL, CLR_DENSACC, CLR_VEL, CLR_VELACC, CLR_VELRGB, CLR_NONE = range(7)
ACC_OFF, ACC_BOX, ACC_CYLY, ACC_CYLYSM = range(4)
NUM_ACC = 4


class Float3(ctypes.Structure):
    _fields_ = [("x", ctypes.c_float), ("y", ctypes.c_float), ("z", ctypes.c_float)]

    def __iter__(self):
        return iter((self.x, self.y, self.z))

    def set(self, v):
        self.x, self.y, self.z = (float(c) for c in v)


class UInt3(ctypes.Structure):
    _fields_ = [("x", ctypes.c_uint32), ("y", ctypes.c_uint32), ("z", ctypes.c_uint32)]

    def __iter__(self):
        return iter((self.x, self.y, self.z))


class Int3(ctypes.Structure):
    _fields_ = [("x", ctypes.c_int32), ("y", ctypes.c_int32), ("z", ctypes.c_int32)]


class Float4(ctypes.Structure):
    # 16-byte aligned in C; in SimParams it already falls on offset 208.
    _fields_ = [("x", ctypes.c_float), ("y", ctypes.c_float), ("z", ctypes.c_float),
                ("w", ctypes.c_float)]


class Accel(ctypes.Structure):
    _fields_ = [("pos", Float3), ("size", Float3), ("acc", Float3), ("type", ctypes.c_uint32)]


class SimParams(ctypes.Structure):
    _fields_ = [
        ("timeStep", ctypes.c_float),
        ("numParticles", ctypes.c_uint32), ("maxParInCell", ctypes.c_uint32),
        ("gravity", Float3), ("globalDamping", ctypes.c_float),
        ("gridSize", UInt3), ("cellSize", Float3),
        ("gridSize_yx", ctypes.c_uint32), ("numCells", ctypes.c_uint32),
        ("worldMin", Float3), ("worldMax", Float3), ("worldSize", Float3),
        ("worldMinD", Float3), ("worldMaxD", Float3), ("worldSizeD", Float3),
        ("particleR", ctypes.c_float), ("h", ctypes.c_float), ("h2", ctypes.c_float),
        ("SpikyKern", ctypes.c_float), ("LapKern", ctypes.c_float), ("Poly6Kern", ctypes.c_float),
        ("particleMass", ctypes.c_float), ("restDensity", ctypes.c_float),
        ("stiffness", ctypes.c_float), ("viscosity", ctypes.c_float),
        ("minDens", ctypes.c_float), ("minDist", ctypes.c_float),
        ("distBndHard", ctypes.c_float), ("distBndSoft", ctypes.c_float),
        ("bndDamp", ctypes.c_float), ("bndStiff", ctypes.c_float), ("bndDampC", ctypes.c_float),
        ("bndType", ctypes.c_uint32), ("bndEffZ", ctypes.c_uint32),
        ("collPos", Float4), ("collR", ctypes.c_float),
        ("spring", ctypes.c_float), ("damping", ctypes.c_float), ("shear", ctypes.c_float),
        ("clrType", ctypes.c_uint32), ("iHue", ctypes.c_int32),
        ("brightness", ctypes.c_float), ("contrast", ctypes.c_float),
        ("dyeType", ctypes.c_int32), ("dyeClear", ctypes.c_int32),
        ("dyeFade", ctypes.c_float), ("dyePos", Float3), ("dyeSize", Float3),
        ("acc", Accel * NUM_ACC), ("iHmap", ctypes.c_int32),
        ("angOut", ctypes.c_float), ("hClose", ctypes.c_float), ("radIn", ctypes.c_float),
        ("rVexit", ctypes.c_float), ("rDexit", ctypes.c_float),
        ("s1", ctypes.c_float), ("s2", ctypes.c_float), ("s3", ctypes.c_float),
        ("s4", ctypes.c_float), ("s5", ctypes.c_float), ("s6", ctypes.c_float),
        ("rAngle", ctypes.c_float), ("rTwist", ctypes.c_float),
        ("rotType", ctypes.c_int32), ("rotBlades", ctypes.c_int32),
        ("rotSize", Int3), ("rotR", ctypes.c_float), ("rotSpc", ctypes.c_float),
        ("r2Dist", ctypes.c_float), ("r2Angle", ctypes.c_float), ("r2twist", ctypes.c_float),
        ("ff2", ctypes.c_float),
        ("_tail", ctypes.c_uint8 * 8),  # sizeof rounds up to the float4 alignment
    ]

    def to_bytes(self) -> bytes:
        return ctypes.string_at(ctypes.addressof(self), ctypes.sizeof(self))

    @classmethod
    def from_bytes(cls, b: bytes) -> "SimParams":
        if len(b) != ctypes.sizeof(cls):
            raise ValueError(f"SimParams is {ctypes.sizeof(cls)} bytes, got {len(b)}")
        return cls.from_buffer_copy(b)

    def copy(self) -> "SimParams":
        return SimParams.from_bytes(self.to_bytes())


_EXPECTED = {"gravity": 12, "gridSize": 28, "numCells": 56, "worldMin": 60, "particleR": 132,
             "bndType": 200, "collPos": 208, "clrType": 240, "acc": 292, "iHmap": 452,
             "rotSize": 516, "ff2": 548}
for _name, _off in _EXPECTED.items():
    assert getattr(SimParams, _name).offset == _off, (_name, getattr(SimParams, _name).offset)
assert ctypes.sizeof(SimParams) == 560, ctypes.sizeof(SimParams)
