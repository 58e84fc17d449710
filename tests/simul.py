"""Synthetic off-axis hologram stacks for the reconstruction path.

Plays the role of the reference's hologram simulator (Simul_holo): a phantom's
analytic 3D Fourier transform is sampled on each illumination's Ewald cap
(the forward counterpart of the cap mapping, cf. Simul_holo/src/fonctions.cpp
calcHolo), turned into a Born (1 + u) or Rytov (exp(u)) field, mixed with a
tilted reference wave into an off-axis hologram, and quantised with shot and
read noise to 12-bit samples stored as uint16.

Conventions follow the reference programs:
  * CIRCLE_CX/CY are absolute coordinates of the +1 order in the fftshifted
    hologram spectrum; the crop is [C-NXMAX, C+NXMAX) in each axis.
  * Illumination tilts are integer spectrum offsets (tx, ty) from the crop
    centre, on a Fermat spiral out to 0.9 NXMAX, so the specular position in
    the crop is (NXMAX+tx, NXMAX+ty).
  * The Ewald radius in spectrum pixels is round(NXMAX*n0/NA).

Everything is computed with torch so that large stacks can be generated on
the GPU; the result is deterministic for a given seed and device.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field, replace

import numpy as np
import torch


@dataclass
class Acquisition:
    """Keys of config_manip.txt / recon.txt that the path reads."""
    ccd_roix: int = 512          # CCD_ROIX: hologram side H
    nxmax: int = 64              # NXMAX: crop half width N (fields are 2N x 2N)
    circle_cx: int = 128         # CIRCLE_CX
    circle_cy: int = 128         # CIRCLE_CY
    dim_final: int = 256         # DIM_FINAL: reconstructed volume side D
    nb_holo: int = 100           # NB_HOLO
    na: float = 1.40             # NA
    n0: float = 1.515            # N0
    lambda0: float = 633e-9      # LAMBDA (m)
    f_tube: float = 0.2          # F_TUBE (m)
    f_obj: float = 0.002         # F_OBJ (m)
    tpcam: float = 1.0e-5        # TPCAM (m): 100 nm per hologram pixel with Gt = 100
    rf: float = 1.0              # RF
    born: int = 1                # BORN (1 Born, 0 Rytov)
    c_aber: int = 1              # C_ABER
    deroul: int = 1              # DEROUL
    volkov: int = 1              # VOLKOV
    nb_threads: int = 4          # NB_THREADS
    export_otf: int = 1          # EXPORT_OTF
    coef_na_obj_limit: float = 1.0  # COEF_NA_OBJ_LIMIT

    @property
    def F(self) -> int:
        return 2 * self.nxmax

    @property
    def rayon(self) -> float:
        n0 = float(np.float32(self.n0))
        na = float(np.float32(self.na))
        return float(np.round(self.nxmax * n0 / na))

    def recon_txt(self) -> str:
        return (
            "# recon.txt\n"
            f"CCD_ROIX {self.ccd_roix}\nDEROUL {self.deroul}\nVOLKOV {self.volkov}\nC_ABER {self.c_aber}\n"
            f"BORN {self.born}\nNB_THREADS {self.nb_threads}\nPREMIER_ANGLE 0\nDIM_FINAL {self.dim_final}\n"
            f"EXPORT_OTF {self.export_otf}\nCOEF_NA_OBJ_LIMIT {self.coef_na_obj_limit}\n"
        )

    def config_manip_txt(self) -> str:
        return (
            "# config_manip.txt\n"
            f"NA {self.na}\nN0 {self.n0}\nLAMBDA {self.lambda0:.10f}\nF_TUBE {self.f_tube}\nF_OBJ {self.f_obj}\n"
            f"TPCAM {self.tpcam:.10f}\nRF {self.rf}\nNXMAX {self.nxmax}\nCIRCLE_CX {self.circle_cx}\n"
            f"CIRCLE_CY {self.circle_cy}\nDIM_ROI {self.ccd_roix}\nNB_HOLO {self.nb_holo}\n"
        )


@dataclass
class Ellipsoid:
    center: tuple          # (x, y, z) in units of the field of view
    semi_axes: tuple       # (a, b, c) in units of the field of view
    dn: float              # real index contrast
    kappa: float = 0.0     # absorption (imaginary index contrast)
    smooth: bool = False   # Gaussian profile (sigma = semi-axis / 2) instead of a uniform body


@dataclass
class Phantom:
    objects: list = field(default_factory=list)
    phase_max: float | None = None   # rescale so the normal-incidence phase peaks here (rad)
    logamp_max: float = 0.1          # bound on |log amplitude| when phase_max rescales the field


# Named workloads: the configurations the path is quoted on.
def workload(name: str) -> tuple[Acquisition, Phantom, int]:
    """Returns (acquisition, phantom, seed) for a named workload."""
    if name == "plain_512_born":      # 100 x 512^2, NXMAX 64, 256^3, Born
        acq = Acquisition(ccd_roix=512, nxmax=64, circle_cx=128, circle_cy=128, dim_final=256,
                          nb_holo=100, born=1)
        ph = Phantom([Ellipsoid((0, 0, 0), (3e-6 / 51.2e-6,) * 3, 0.02)])
        return acq, ph, 0
    if name == "rytov_1024":          # 600 x 1024^2, NXMAX 128, 512^3, Rytov, <= 40 rad
        acq = Acquisition(ccd_roix=1024, nxmax=128, circle_cx=256, circle_cy=256, dim_final=512,
                          nb_holo=600, born=0)
        ph = Phantom([
            Ellipsoid((-0.05, 0.02, 0.0), (0.22, 0.17, 0.15), 0.03, 0.003, smooth=True),
            Ellipsoid((0.06, -0.04, 0.02), (0.16, 0.21, 0.14), 0.05, 0.005, smooth=True),
            Ellipsoid((0.01, 0.07, -0.02), (0.14, 0.12, 0.12), 0.01, 0.0, smooth=True),
        ], phase_max=40.0)
        return acq, ph, 1
    if name == "tomo_config_1024":    # the reference's Tomo_config: 500 x 1024^2, NXMAX 125, CIRCLE 247,777, 512^3
        acq = Acquisition(ccd_roix=1024, nxmax=125, circle_cx=247, circle_cy=777, dim_final=512, nb_holo=500,
                          na=1.40, n0=1.515, lambda0=632e-9, f_tube=0.15, f_obj=0.002, tpcam=5.5e-6, rf=0.75,
                          born=0)
        ph = Phantom([
            Ellipsoid((-0.05, 0.02, 0.0), (0.22, 0.17, 0.15), 0.03, 0.003, smooth=True),
            Ellipsoid((0.06, -0.04, 0.02), (0.16, 0.21, 0.14), 0.05, 0.005, smooth=True),
        ], phase_max=30.0)
        return acq, ph, 5
    if name == "large_2048":          # 1000 x 2048^2, NXMAX 256, 1024^3
        acq = Acquisition(ccd_roix=2048, nxmax=256, circle_cx=512, circle_cy=512, dim_final=1024,
                          nb_holo=1000, born=1)
        rng = np.random.default_rng(4)
        objs = []
        for _ in range(200):
            r = rng.uniform(0.5e-6, 4e-6) / 204.8e-6
            c = tuple(rng.uniform(-0.3, 0.3, 3))
            objs.append(Ellipsoid(c, (r, r, r), float(rng.uniform(0.005, 0.04))))
        return acq, Phantom(objs), 4
    raise KeyError(name)


def small_workload(name: str, **over) -> tuple[Acquisition, Phantom, int]:
    acq, ph, seed = workload(name)
    return replace(acq, **over), ph, seed


def spiral_tilts(M: int, nxmax: int, frac: float = 0.9) -> np.ndarray:
    """Integer tilt offsets (tx, ty) on a Fermat spiral inside frac*NXMAX."""
    golden = math.pi * (3.0 - math.sqrt(5.0))
    k = np.arange(M, dtype=np.float64)
    r = frac * nxmax * np.sqrt((k + 0.5) / max(M, 1))
    th = k * golden
    t = np.stack([np.round(r * np.cos(th)), np.round(r * np.sin(th))], 1).astype(np.int64)
    lim = int(math.floor(frac * nxmax))
    return np.clip(t, -lim, lim)


def _sphere_ft(rho: torch.Tensor) -> torch.Tensor:
    """3 (sin r - r cos r) / r^3 (unit-volume ball transform, 1 at r = 0)."""
    small = rho.abs() < 1e-3
    r = torch.where(small, torch.ones_like(rho), rho)
    v = 3.0 * (torch.sin(r) - r * torch.cos(r)) / r ** 3
    return torch.where(small, 1.0 - rho * rho / 10.0, v)


def _phantom_ft(ph: Phantom, qx, qy, qz) -> torch.Tensor:
    """Complex index-contrast transform at spatial frequencies q (cycles/FOV)."""
    out = torch.zeros(qx.shape, dtype=torch.complex128, device=qx.device)
    for e in ph.objects:
        a, b, c = e.semi_axes
        ramp = torch.exp(-2j * math.pi * (qx * e.center[0] + qy * e.center[1] + qz * e.center[2]))
        if e.smooth:  # Gaussian body, sigma = semi-axis / 2
            sa, sb, sc = a / 2, b / 2, c / 2
            g = torch.exp(-2 * math.pi ** 2 * ((sa * qx) ** 2 + (sb * qy) ** 2 + (sc * qz) ** 2))
            out = out + complex(e.dn, e.kappa) * (2 * math.pi) ** 1.5 * sa * sb * sc * g * ramp
        else:
            rho = 2 * math.pi * torch.sqrt((a * qx) ** 2 + (b * qy) ** 2 + (c * qz) ** 2)
            vol = 4.0 / 3.0 * math.pi * a * b * c
            out = out + complex(e.dn, e.kappa) * vol * _sphere_ft(rho) * ramp
    return out


def cap_fields(acq: Acquisition, ph: Phantom, tilts: np.ndarray, device="cpu") -> torch.Tensor:
    """Complex Born/Rytov phase u (M x F x F, centred field grid) per tilt."""
    N, F = acq.nxmax, acq.F
    r = acq.rayon
    f = torch.arange(-N, N, device=device, dtype=torch.float64)
    fy, fx = torch.meshgrid(f, f, indexing="ij")
    fd2 = fx * fx + fy * fy
    inside = fd2 < N * N
    s = torch.sqrt(torch.clamp(r * r - fd2, min=0.0))
    out = torch.empty((len(tilts), F, F), dtype=torch.complex128, device=device)
    scale = None
    for i, (tx, ty) in enumerate(tilts):
        sz0 = math.sqrt(max(r * r - tx * tx - ty * ty, 0.0))
        V = _phantom_ft(ph, fx - tx, fy - ty, s - sz0)
        S = torch.where(inside, 1j * V * r / torch.clamp(s, min=1.0), torch.zeros_like(V))
        # centred spectrum -> centred field (object at the field centre)
        u = torch.fft.fftshift(torch.fft.ifft2(torch.fft.ifftshift(S))) * (F * F)
        out[i] = u
    # global scale: normal-incidence phase peak; the log amplitude is scaled
    # separately so that it stays within +-logamp_max
    if ph.phase_max is not None:
        V0 = _phantom_ft(ph, fx, fy, s - r)
        S0 = torch.where(inside, 1j * V0 * r / torch.clamp(s, min=1.0), torch.zeros_like(V0))
        u0 = torch.fft.fftshift(torch.fft.ifft2(torch.fft.ifftshift(S0))) * (F * F)
        s_im = ph.phase_max / float(u0.imag.abs().max())
        s_re = min(s_im, ph.logamp_max / max(float(out.real.abs().max()), 1e-30))
        return torch.complex(out.real * s_re, out.imag * s_im)
    else:
        # physical scaling for weak objects: phase ~ k0 * dn * thickness
        fov = acq.ccd_roix * (acq.tpcam * acq.rf / (acq.f_tube / acq.f_obj))
        k0 = 2 * math.pi / acq.lambda0
        V0 = _phantom_ft(ph, fx * 0, fy * 0, fx * 0)[0, 0]
        # the transform at q = 0 integrates the index over the unit FOV volume
        u_mean = float(out[:, N, N].imag.abs().max()) if len(tilts) else 1.0
        vol_phase = max(abs(e.dn) * 2 * max(e.semi_axes) * fov * k0 for e in ph.objects)
        scale = vol_phase / max(u_mean, 1e-30)
        del V0
    return out * scale


def holograms(acq: Acquisition, ph: Phantom, M: int | None = None, seed: int = 0, device="cpu",
              mean_e: float = 2000.0, read_sigma: float = 3.0, bits: int = 12, ref_fraction: float = 0.7,
              tilts: np.ndarray | None = None) -> dict:
    """Generates M off-axis holograms (uint16, M x H x H) and the aberration mask."""
    M = acq.nb_holo if M is None else M
    H, N, F = acq.ccd_roix, acq.nxmax, acq.F
    if tilts is None:
        tilts = spiral_tilts(M, N)
    g = torch.Generator(device=device)
    g.manual_seed(int(seed))
    u = cap_fields(acq, ph, tilts, device=device)
    ratio = torch.exp(u) if acq.born == 0 else 1.0 + u
    # band-limited upsampling of the F x F field ratio to the H x H camera grid
    holos = torch.empty((M, H, H), dtype=torch.uint16, device=device)
    yy = torch.arange(H, device=device, dtype=torch.float64)
    Y, X = torch.meshgrid(yy, yy, indexing="ij")
    # reference / object intensity split of the 2000 e- mean (fringe visibility < 1 keeps the
    # 12-bit range unclipped)
    a_r = math.sqrt(mean_e * ref_fraction)
    a_o = math.sqrt(mean_e * (1.0 - ref_fraction))
    pad = (H - F) // 2
    for i, (tx, ty) in enumerate(tilts):
        spec = torch.fft.fftshift(torch.fft.fft2(torch.fft.ifftshift(ratio[i])))
        big = torch.zeros((H, H), dtype=torch.complex128, device=device)
        big[pad:pad + F, pad:pad + F] = spec
        gH = torch.fft.fftshift(torch.fft.ifft2(torch.fft.ifftshift(big))) * (H * H) / (F * F)
        fcx = acq.circle_cx - H // 2 + int(tx)
        fcy = acq.circle_cy - H // 2 + int(ty)
        carrier = torch.exp(2j * math.pi * (fcx * X + fcy * Y) / H)
        inten = a_r * a_r + a_o * a_o * gH.abs() ** 2 + 2 * a_r * a_o * (carrier * gH).real
        inten = torch.clamp(inten, min=0.0)
        noisy = torch.poisson(inten.float(), generator=g).double()
        noisy = noisy + read_sigma * torch.randn(noisy.shape, generator=g, device=device, dtype=torch.float64)
        holos[i] = torch.clamp(torch.round(noisy), 0, 2 ** bits - 1).to(torch.int32).to(torch.uint16)
    # aberration mask: background 255, dilated object support 0 (field grid)
    supp = (u.imag.abs().amax(0) > 0.05 * float(u.imag.abs().max())) if M else torch.zeros((F, F), dtype=torch.bool)
    k = max(1, F // 32)
    dil = torch.nn.functional.max_pool2d(supp.float()[None, None], 2 * k + 1, 1, k)[0, 0] > 0
    mask = torch.where(dil, torch.zeros((F, F), dtype=torch.uint8, device=device),
                       torch.full((F, F), 255, dtype=torch.uint8, device=device))
    return {"holos": holos, "tilts": tilts, "mask": mask, "u": u}
