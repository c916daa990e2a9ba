"""The benchmark workloads as run descriptors.

Mapping of a channel workload to the reference's parameters (the reference
ties them to its square side L, src/mpi_LBM_GK_pops_perturb.cpp:144-150):
L := square side s, T0 = s/u0, dt = 1/T0, F0 = u0^2 s / 2 (drag normalised by
F0), beta0 = s u0^2 / ((W-1)(H-1)) (the reference's formula with its Dx, Dy
generalised to W, H), alpha = k.  ZERO_MEAN's constant 1.775 is calibrated for
the reference's own geometry only, so these channel workloads use shift 0.
Square: side s centred at (xc, yc): xmin = xc - floor(s/2), xmax = xmin + s,
likewise in y; where s = H/5 is not an integer it is rounded down.
"""
from __future__ import annotations

from dataclasses import dataclass, field

from . import RunDesc, PERTURB_UNIFORM, RESAMPLE_REFERENCE, FP32, FP64


@dataclass
class Run:
    width: int
    height: int
    side: int
    xc: int
    yc: int
    nclones: int
    u0: float
    tau: float
    k: float
    noise: float
    seed: int
    perturb_mode: int = PERTURB_UNIFORM
    resample_mode: int = RESAMPLE_REFERENCE
    # random body-force field of the forcing variant (0 steps: none)
    field_steps: int = 0
    field_eps: float = 0.0
    field_sigma: float = 32.0

    @property
    def xmin(self):
        return self.xc - self.side // 2

    @property
    def ymin(self):
        return self.yc - self.side // 2

    @property
    def beta(self):
        return self.side * self.u0 * self.u0 / ((self.width - 1) * (self.height - 1))

    @property
    def F0(self):
        return self.u0 * self.u0 * self.side * 0.5

    @property
    def dt(self):
        return self.u0 / self.side

    @property
    def nodes(self):
        return self.width * self.height

    def desc(self, run_index: int = 0) -> RunDesc:
        return RunDesc(width=self.width, height=self.height, xmin=self.xmin,
                       xmax=self.xmin + self.side, ymin=self.ymin, ymax=self.ymin + self.side,
                       nclones=self.nclones, ranks=1, tau=self.tau, beta=self.beta,
                       alpha=self.k, force_scale=1.0 / self.F0, force_shift=0.0, dt=self.dt,
                       perturb_mode=self.perturb_mode, resample_mode=self.resample_mode,
                       eps=self.noise, seed=self.seed, nsnap=0,
                       field_mode=1 if self.field_steps > 0 else 0, field_steps=self.field_steps,
                       field_eps=self.field_eps, field_sigma=self.field_sigma)


@dataclass
class Workload:
    name: str
    runs: list[Run]
    steps: int          # LB steps per cloning interval (T)
    intervals: int      # cloning steps
    precision: int
    init_noise: float = 1e-3
    notes: str = ""

    @property
    def lattice_updates_per_interval(self) -> int:
        return sum(r.nclones * r.nodes for r in self.runs) * self.steps

    def descs(self) -> list[RunDesc]:
        return [r.desc(i) for i, r in enumerate(self.runs)]


def c1() -> Workload:
    return Workload("c1_plain_fp64_16x200x50",
                    [Run(200, 50, 8, 50, 25, 16, 0.05, 0.56, 0.1, 1e-4, 1)], 100, 20, FP64)


def c2(precision: int = FP64) -> Workload:
    return Workload(f"c2_512x400x100_{'fp64' if precision == FP64 else 'fp32'}",
                    [Run(400, 100, 20, 100, 50, 512, 0.05, 0.53, k, 1e-4, 2) for k in (-0.2, 0.2)],
                    200, 50, precision)


def c3() -> Workload:
    return Workload("c3_4096x256x64_fp32",
                    [Run(256, 64, 12, 64, 32, 4096, 0.04, 0.55, 0.3, 1e-5, 3)], 100, 100, FP32)


def c4() -> Workload:
    sizes = [(128, 32), (192, 48), (256, 64), (320, 80), (384, 96), (448, 112), (512, 128), (256, 128)]
    runs = [Run(w, h, h // 5, w // 4, h // 2, 256, 0.05, 0.55, -0.5 + i / 7, 1e-5, 4)
            for i, (w, h) in enumerate(sizes)]
    return Workload("c4_uneven_8x256", runs, 100, 40, FP32)


def c3_forcing() -> Workload:
    """The forcing variant on the 4096-clone 256x64 channel: every clone draws
    a Gaussian random body-force field (covariance exp(-r^2/(2 sigma^2)),
    sigma = 32 as in the reference, amplitude eps = 0.1) at the start of each
    interval and steps its first 20 of the 100 steps under it
    (src/mpi_LBM_GK_forcing.cpp:333-364)."""
    return Workload("c3f_4096x256x64_fp32_forcing",
                    [Run(256, 64, 12, 64, 32, 4096, 0.04, 0.55, 0.3, 1e-5, 3,
                         field_steps=20, field_eps=0.1, field_sigma=32.0)], 100, 100, FP32)


def c3_forcing_small() -> Workload:
    """256 clones of the forcing workload: the case the ncu captures of the
    random-field kernels run on."""
    return Workload("c3fs_256x256x64_fp32_forcing",
                    [Run(256, 64, 12, 64, 32, 256, 0.04, 0.55, 0.3, 1e-5, 3,
                         field_steps=20, field_eps=0.1, field_sigma=32.0)], 100, 100, FP32)


def c3_small() -> Workload:
    """256 clones of the c3 lattice (151 MB per FP32 buffer, above L2): the
    case the ncu captures of the step kernel run on."""
    return Workload("c3s_256x256x64_fp32",
                    [Run(256, 64, 12, 64, 32, 256, 0.04, 0.55, 0.3, 1e-5, 3)], 100, 100, FP32)


def c3_medium() -> Workload:
    """1024 clones of the c3 lattice (604 MB per FP32 buffer, 4.7x L2): the
    case the DRAM-traffic capture of the step kernel runs on."""
    return Workload("c3m_1024x256x64_fp32",
                    [Run(256, 64, 12, 64, 32, 1024, 0.04, 0.55, 0.3, 1e-5, 3)], 100, 100, FP32)


def c2_fp32() -> Workload:
    return c2(FP32)


def c5() -> Workload:
    """Adjoint drag gradient: 64 clones of 400x100, square 20 at (100,50),
    gradient of the drag integrated over T = 200 steps, checkpoints every 20."""
    return Workload("c5_adjoint_64x400x100", [Run(400, 100, 20, 100, 50, 64, 0.05, 0.56, 0.0, 1e-4, 5)],
                    200, 1, FP32)


WORKLOADS = {"c5": c5, "c1": c1, "c2": c2, "c2f32": c2_fp32, "c3": c3, "c3f": c3_forcing, "c3fs": c3_forcing_small, "c3s": c3_small, "c3m": c3_medium, "c4": c4}
