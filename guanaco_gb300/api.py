"""Drop-in for the reference's public Python API on the device path:
``guanaco.correct_projections`` and ``guanaco.reconstruct``
(src/guanaco/__init__.py:27-28), plus the helpers they use.

The helpers that decide numbers -- centres, angular weights, the defocus
slabs -- follow the reference's numpy code step by step, with the same numpy
scalar types, so they produce the same float32 values.  The per-tilt
``corr`` loop and the per-row ``recon`` loop of the reference collapse into
one device pass each (or one pass for both with :func:`reconstruct_ctf`).
"""
from __future__ import annotations

from math import pi

import numpy as np

from . import detail
from .fbp import FbpPlan

__all__ = [
    "correct_projections", "reconstruct", "reconstruct_ctf", "get_centre",
    "compute_angular_weights", "get_weights", "get_defocus_steps", "get_ctf", "get_ctf_array",
]


def _gpu(device):
    if detail.eDevice.convert(device) != detail.eDevice.gpu:
        raise RuntimeError("guanaco_gb300 implements the device path only: pass device='gpu'")


def get_centre(shape, centre, sinogram_order=True):
    """src/guanaco/detail/reconstruct.py:32-52."""
    if not sinogram_order:
        shape = list(shape)
        shape[0], shape[-2] = shape[-2], shape[0]
    if centre is None:
        centre = np.ones(shape[0], dtype="float32") * (shape[-1] * 0.5)
    elif np.array(centre).size == 1:
        centre = np.ones(shape[0], dtype="float32") * centre
    return np.asarray(centre).astype(dtype="float32", copy=False)


def compute_angular_weights(angles):
    """src/guanaco/detail/reconstruct.py:55-105 (interval sums in the dtype of
    ``angles``, as numpy evaluates them there)."""
    angles = np.asarray(angles)
    index = np.argsort(angles)
    weights = np.zeros(angles.size)
    if angles.size > 1:
        mean_interval = abs(angles[index[-1]] - angles[index[0]]) / (angles.size - 1)
        assert mean_interval != 0
    else:
        mean_interval = 1.0
    for i in range(angles.size):
        sum_intervals = 0.0
        sum_weights = 0.0
        if i - 2 >= 0:
            sum_weights += 1.0 / 1.5
            sum_intervals += (1.0 / 1.5) * (angles[index[i - 1]] - angles[index[i - 2]])
        if i - 1 >= 0:
            sum_weights += 2.0
            sum_intervals += 2.0 * (angles[index[i]] - angles[index[i - 1]])
        if i + 1 < angles.size:
            sum_weights += 2.0
            sum_intervals += 2.0 * (angles[index[i + 1]] - angles[index[i]])
        if i + 2 < angles.size:
            sum_weights += 1.0 / 1.5
            sum_intervals += (1.0 / 1.5) * (angles[index[i + 2]] - angles[index[i + 1]])
        if sum_weights != 0:
            weights[index[i]] = sum_intervals / sum_weights
        else:
            weights[index[i]] = 1.0
    weights /= mean_interval
    return weights


def get_weights(angles, angular_weights=False):
    """src/guanaco/detail/reconstruct.py:108-124."""
    if angular_weights:
        return compute_angular_weights(angles)
    return np.ones(np.shape(angles))


def get_defocus_steps(defocus, num_defocus=None, step_defocus=None, width=None, centre=None,
                      pixel_size=None):
    """src/guanaco/detail/correct.py:44-93: (min, max, step, num)."""
    if num_defocus is None or num_defocus <= 0:
        num_defocus = 1
    if num_defocus == 1:
        min_defocus = defocus
        max_defocus = defocus
        step_defocus = 0
    else:
        if step_defocus is not None and step_defocus > 0:
            min_defocus = defocus - 0.5 * (num_defocus - 1) * step_defocus
            max_defocus = defocus + 0.5 * (num_defocus - 1) * step_defocus
        else:
            centre = np.asarray(centre)
            z0 = defocus - centre * pixel_size
            z1 = defocus + centre * pixel_size
            z2 = defocus - (width - centre) * pixel_size
            z3 = defocus + (width - centre) * pixel_size
            min_defocus = min([z0.min(), z1.min(), z2.min(), z3.min()])
            max_defocus = max([z0.max(), z1.max(), z2.max(), z3.max()])
            step_defocus = (max_defocus - min_defocus) / (num_defocus - 1)
    return min_defocus, max_defocus, step_defocus, num_defocus


def slab_defoci(min_defocus, num_defocus, step_defocus):
    """The defocus of every CTF slab exactly as get_ctf_array forms it
    (correct.py:195-199: ``min_defocus + d * step_defocus``)."""
    return np.array([float(min_defocus + d * step_defocus) for d in range(num_defocus)],
                    dtype=np.float64)


def get_ctf(width, height, pixel_size, energy, defocus, spherical_aberration=0, astigmatism=0,
            astigmatism_angle=0, phase_shift=0):
    """src/guanaco/detail/correct.py:116-154 (keV, mm, degrees)."""
    c = detail.CTF(l=detail.get_electron_wavelength(energy * 1000), df=defocus,
                   Cs=spherical_aberration * 1e7, Ca=astigmatism, Pa=astigmatism_angle * pi / 180,
                   phi=phase_shift * pi / 180)
    return c.get_ctf_simple(width, height, pixel_size)


def get_ctf_array(width, height, pixel_size, energy, min_defocus, num_defocus, step_defocus,
                  spherical_aberration=0, astigmatism=0, astigmatism_angle=0, phase_shift=0):
    """src/guanaco/detail/correct.py:157-214 (complex64 (D, H, W))."""
    out = np.zeros((num_defocus, height, width), dtype="complex64")
    for d in range(num_defocus):
        df = min_defocus + d * step_defocus
        out[d] = get_ctf(width, height, pixel_size, energy, df, spherical_aberration,
                         astigmatism, astigmatism_angle, phase_shift)
    return out


def _ctf_setup(projections_shape, centre, pixel_size, defocus, num_defocus, step_defocus):
    T, H, W = projections_shape
    mn, mx, step, nd = get_defocus_steps(defocus, num_defocus, step_defocus, W, centre, pixel_size)
    assert abs(mn + (nd - 1) * step - mx) < 1e-7, "Inconsistent defocus steps"
    return mn, mx, step, nd


def correct_projections(projections, centre=None, pixel_size=1, energy=None, defocus=None,
                        num_defocus=None, step_defocus=None, spherical_aberration=0, astigmatism=0,
                        astigmatism_angle=0, phase_shift=0, corrected_output=None, device="cpu",
                        staging="f32"):
    """src/guanaco/detail/correct.py:217-318: returns (projections, relative
    min defocus, relative max defocus); the corrected stack is (T, D, H, W)
    float32, or (T, H, W) for one slab, unnormalised like the reference."""
    _gpu(device)
    if defocus is None:
        return projections, 0, 0
    proj = np.ascontiguousarray(projections, dtype=np.float32)
    T, H, W = proj.shape
    mn, mx, step, nd = _ctf_setup(proj.shape, centre, pixel_size, defocus, num_defocus,
                                  step_defocus)
    import torch

    plan = FbpPlan(T, H, W, np.zeros(T, np.float32), pixel_size=pixel_size, input="raw",
                   correct=True, num_defocus=nd, slab_defocus=slab_defoci(mn, nd, step),
                   min_defocus=float(mn - defocus) if nd > 1 else 0.0,
                   max_defocus=float(mx - defocus) if nd > 1 else 0.0, energy=energy,
                   spherical_aberration=spherical_aberration, astigmatism=astigmatism,
                   astigmatism_angle=astigmatism_angle, phase_shift=phase_shift)
    try:
        dp = torch.from_numpy(np.require(proj, np.float32, ["C", "W"])).cuda()
        dc = torch.empty((T, nd, H, W), dtype=torch.float32, device="cuda")
        plan.correct(dp, dc)
        out = dc.cpu().numpy()
    finally:
        plan.close()
    if isinstance(corrected_output, str):  # correct.py:96-113: a memory-mapped file
        corrected_output = np.memmap(corrected_output, mode="w+", dtype="float32",
                                     shape=out.shape)
    if corrected_output is not None:
        target = np.asarray(corrected_output).reshape(out.shape)
        target[...] = out
        out = corrected_output.reshape(out.shape)
    if nd == 1:
        out = out.reshape(proj.shape)
    return out, mn - defocus, mx - defocus


def reconstruct(tomogram, angles, reconstruction=None, centre=None, pixel_size=1, min_defocus=0,
                max_defocus=0, sinogram_order=False, transform=None, angular_weights=False,
                device="cpu", ncore=None, nchunk=None, gpu_list=None, staging="f32"):
    """src/guanaco/detail/reconstruct.py:127-213 on the device: the whole
    stack in one pass instead of one ``recon`` call per row.

    Accepts (THETA, Y, X), (Y, THETA, X), (THETA, D, Y, X) or (Y, D, THETA, X)
    as the reference does; returns the (Y, X, X) float32 volume.  With
    ``gpu_list`` the Y rows are split into len(gpu_list) contiguous bands
    (sizes as the reference's get_ncore_slices, mp.py:9-35, each edge moved to
    the next even row) and band i runs on device gpu_list[i], all bands at
    once (mp.py:61-66, 86-101): rows are independent once the projections are
    corrected, so no exchange is needed.
    ``ncore`` and ``nchunk`` only split the reference's per-row Python loop and
    are accepted and ignored."""
    _gpu(device)
    t = np.asarray(tomogram)
    assert len(t.shape) in [3, 4], "Dimensions must be 3 or 4"
    t = t.astype("float32", copy=False)
    if sinogram_order:
        t = np.swapaxes(t, 0, -2)  # to (THETA, [D,] Y, X)
    t = np.ascontiguousarray(t)
    T, H, W = t.shape[0], t.shape[-2], t.shape[-1]
    D = t.shape[1] if t.ndim == 4 else 1
    if reconstruction is None:
        reconstruction = np.zeros((H, W, W), dtype="float32")
    else:
        assert reconstruction.shape[0] == H, "Inconsistent reconstruction/sinogram shape"
        assert reconstruction.shape[1] == W, "Inconsistent reconstruction/sinogram shape"
        assert reconstruction.shape[2] == W, "Inconsistent reconstruction/sinogram shape"
    centre = get_centre((H, T, W), centre)
    weights = get_weights(np.asarray(angles), angular_weights)

    def run_band(y0, y1):
        band = np.ascontiguousarray(t[..., y0:y1, :])
        plan = FbpPlan(T, y1 - y0, W, angles, grid_height=W, grid_width=W,
                       centre=centre[y0:y1], pixel_size=pixel_size,
                       input="corrected" if t.ndim == 4 else "raw", correct=False,
                       num_defocus=D, min_defocus=min_defocus, max_defocus=max_defocus,
                       weights=weights, minus=(transform == "minus"), staging=staging)
        try:
            reconstruction[y0:y1] = plan.execute_host(band)
        finally:
            plan.close()

    if not gpu_list:
        run_band(0, H)
        return reconstruction
    # band edges on even rows: the filter transforms rows in pairs, so a pair
    # never straddles two bands and the volume is the unsplit one bit for bit
    bands = [(min(H, y0 + (y0 & 1)), min(H, y1 + (y1 & 1))) for y0, y1 in row_bands(H, len(gpu_list))]
    import concurrent.futures as cf

    import torch

    def worker(gpu, y0, y1):
        torch.cuda.set_device(int(gpu))  # this thread's current device
        run_band(y0, y1)

    with cf.ThreadPoolExecutor(len(bands)) as ex:
        for f in [ex.submit(worker, g, y0, y1) for g, (y0, y1) in zip(gpu_list, bands)
                  if y1 > y0]:
            f.result()
    return reconstruction


def row_bands(nrows, nbands):
    """Contiguous row bands of sizes nrows // nbands, the first nrows % nbands
    one row larger (get_ncore_slices, src/guanaco/detail/mp.py:9-35)."""
    size, extra = divmod(int(nrows), int(nbands))
    bands, y0 = [], 0
    for i in range(int(nbands)):
        y1 = y0 + size + (1 if i < extra else 0)
        bands.append((y0, y1))
        y0 = y1
    return bands


def reconstruct_ctf(projections, angles, centre=None, pixel_size=1, energy=300, defocus=None,
                    num_defocus=None, step_defocus=None, spherical_aberration=0, astigmatism=0,
                    astigmatism_angle=0, phase_shift=0, transform=None, angular_weights=False,
                    grid_height=None, staging="f32", device="gpu"):
    """correct_projections followed by reconstruct (the reference's
    ``reconstruct_file`` with method FBP_CTF, reconstruct.py:336-400) in one
    device pass: the corrected stack never leaves the GPU."""
    _gpu(device)
    proj = np.ascontiguousarray(projections, dtype=np.float32)
    T, H, W = proj.shape
    c = get_centre(proj.shape, centre, False)
    weights = get_weights(np.asarray(angles), angular_weights)
    Z = W if grid_height is None else int(grid_height)
    if defocus is None:
        plan = FbpPlan(T, H, W, angles, grid_height=Z, grid_width=W, centre=c,
                       pixel_size=pixel_size, input="raw", correct=False, weights=weights,
                       minus=(transform == "minus"), staging=staging)
    else:
        mn, mx, step, nd = _ctf_setup(proj.shape, c, pixel_size, defocus, num_defocus,
                                      step_defocus)
        plan = FbpPlan(T, H, W, angles, grid_height=Z, grid_width=W, centre=c,
                       pixel_size=pixel_size, input="raw", correct=True, num_defocus=nd,
                       slab_defocus=slab_defoci(mn, nd, step), min_defocus=float(mn - defocus),
                       max_defocus=float(mx - defocus), energy=energy,
                       spherical_aberration=spherical_aberration, astigmatism=astigmatism,
                       astigmatism_angle=astigmatism_angle, phase_shift=phase_shift,
                       weights=weights, minus=(transform == "minus"), staging=staging)
    try:
        return plan.execute_host(proj)
    finally:
        plan.close()


# ------------------------------------------------------------------ MRC files
def _read_projection_metadata(infile):
    """Angles (rad, float32) from the FEI1 "Alpha tilt" records, the voxel size,
    and for a corrected stack the relative defocus range from the "Defocus"
    records (reconstruct.py:248-304)."""
    from . import mrc

    ang = mrc.fei1_angles_deg(infile)
    assert infile.data.shape[0] == ang.shape[0], "Inconsistent data/header shape"
    angles = np.deg2rad(ang).astype(np.float32)
    if infile.data.ndim == 4:
        df = mrc.fei1_defocus(infile).astype(np.float32)
        assert infile.data.shape[1] == df.shape[0], "Inconsistent data/header shape"
        return angles, infile.voxel_size, float(np.min(df)), float(np.max(df))
    return angles, infile.voxel_size, 0, 0


def reconstruct_file(input_filename, output_filename, corrected_filename="GUANACO_CORRECTED.dat",
                     start_angle=None, step_angle=None, pixel_size=None, centre=None, energy=None,
                     defocus=None, num_defocus=None, step_defocus=None, spherical_aberration=None,
                     astigmatism=None, astigmatism_angle=None, phase_shift=None, device="cpu",
                     ncore=None, transform=None, angular_weights=False, chunk_size=None,
                     method="FBP_CTF", num_iter=None, staging="f32"):
    """src/guanaco/detail/reconstruct.py:216-402 on the device.

    Reads an MRC tilt series (T, H, W) -- or an already corrected stack
    (T, D, H, W) -- with its angles (FEI1 "Alpha tilt") and voxel size unless
    ``start_angle``, ``step_angle`` and ``pixel_size`` are all given, and writes
    the (H, W, W) float32 volume with the same voxel size.  Raw projections
    with a ``defocus`` are corrected and reconstructed in one device pass; the
    corrected stack stays on the GPU, so ``corrected_filename`` is not written
    (``correct_file`` writes it).  Only the FBP_CTF method is provided (the
    reference hands the others to tomopy)."""
    from . import mrc

    _gpu(device)
    if method != "FBP_CTF":
        raise RuntimeError(f"reconstruct_file: method {method!r} is not provided here "
                           "(only FBP_CTF; the reference delegates the others to tomopy)")
    infile = mrc.open_mrc(input_filename)
    projections = infile.data
    if start_angle is None or step_angle is None or pixel_size is None:
        angles, voxel_size, min_defocus, max_defocus = _read_projection_metadata(infile)
        assert voxel_size["x"] == voxel_size["y"], "Pixel must be a square"
        pixel_size = voxel_size["x"]
        voxel = (voxel_size["x"], voxel_size["y"], voxel_size["z"])
    else:
        angles = np.deg2rad(start_angle + np.arange(projections.shape[0]) * step_angle)
        angles = angles.astype(np.float32)
        voxel = pixel_size
        min_defocus = max_defocus = 0
    H, W = projections.shape[-2], projections.shape[-1]
    centre = get_centre(projections.shape, centre, False)
    if projections.ndim == 4:
        volume = reconstruct(np.asarray(projections), angles, None, centre, pixel_size,
                             min_defocus, max_defocus, False, transform, angular_weights,
                             device=device, staging=staging)
    else:
        volume = reconstruct_ctf(np.asarray(projections), angles, centre, pixel_size,
                                 energy=energy, defocus=defocus, num_defocus=num_defocus,
                                 step_defocus=step_defocus,
                                 spherical_aberration=spherical_aberration or 0,
                                 astigmatism=astigmatism or 0,
                                 astigmatism_angle=astigmatism_angle or 0,
                                 phase_shift=phase_shift or 0, transform=transform,
                                 angular_weights=angular_weights, staging=staging,
                                 device=device)
    with mrc.new_mrc(output_filename, (H, W, W), np.float32, voxel) as outfile:
        outfile.data[...] = volume
    return volume


def correct_file(input_filename, output_filename, centre=None, energy=None, defocus=None,
                 num_defocus=None, step_defocus=None, spherical_aberration=None, astigmatism=None,
                 astigmatism_angle=None, phase_shift=None, device="cpu"):
    """src/guanaco/detail/correct.py:321-473 on the device: the corrected
    stack (T, D, H, W) with FEI1 records carrying each image's tilt and
    relative defocus."""
    from . import mrc

    _gpu(device)
    infile = mrc.open_mrc(input_filename)
    ang = mrc.fei1_angles_deg(infile)
    assert infile.data.shape[0] == ang.shape[0], "Inconsistent data/header array shape"
    angles = np.deg2rad(ang).astype(np.float32)
    voxel_size = infile.voxel_size
    assert voxel_size["x"] == voxel_size["y"]
    pixel_size = voxel_size["x"]
    projections = np.asarray(infile.data)
    centre = get_centre(projections.shape, centre, False)
    if num_defocus is None or num_defocus == 0:
        num_defocus = 1
        step_defocus = 0
    shape = (projections.shape[0], num_defocus, projections.shape[1], projections.shape[2])
    with mrc.new_mrc(output_filename, shape, np.float32,
                     (voxel_size["x"], voxel_size["y"], voxel_size["z"]), fei1=True) as outfile:
        _, min_defocus, max_defocus = correct_projections(
            projections, centre, pixel_size, energy, defocus, num_defocus, step_defocus,
            spherical_aberration or 0, astigmatism or 0, astigmatism_angle or 0,
            phase_shift or 0, outfile.data, device)
        if step_defocus is None:
            step_defocus = 0 if num_defocus == 1 else (max_defocus - min_defocus) / (num_defocus - 1)
        for j in range(shape[0]):
            for i in range(shape[1]):
                outfile.extended_header[j, i]["Alpha tilt"] = np.rad2deg(angles[j])
                outfile.extended_header[j, i]["Defocus"] = min_defocus + i * step_defocus
