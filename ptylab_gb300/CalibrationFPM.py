"""FPM illumination calibration, mirroring PtyLab's ``IlluminationCalibration``
(PtyLab/Reconstruction/CalibrationFPM.py:33-919): the LED positions (and
optionally the pupil radius / NA) are refined from the brightfield frames'
Fourier-domain circle edges before an FPM reconstruction.

The arithmetic runs in libptyg's sm_103a kernels (``ptyg_calib_*``): the
windowed inverse transforms, normalisation and Gaussian smoothing of every
frame, the circle-edge search over radii and grid shifts, and the RMSE of
every candidate shift (one masked inverse transform each).  The reference's
decisions stay on the host in its own order: k-means split of the frames,
candidate selection, edge repeats, the radius iteration, the RANSAC fit and
the encoder update.  The reference treats each LED on its own, so the
search rounds of all LEDs run together, one batch of kernels per round.

Differences from the reference, by design: plotting (``plot = True``,
``plotCalibration``) is not available; frames must be 32, 64, 128 or 256
pixels square (the sizes of the library's transforms); the RANSAC draws come from a fixed-seed generator, so a
calibration is reproducible (scikit-image's draws are unseeded); the k-means
split is two-cluster Lloyd iterations started from the faintest and the
brightest frame (scikit-learn's KMeans starts from random draws).
"""

from __future__ import annotations

import ctypes as C
import logging

import numpy as np

from . import _native

logger = logging.getLogger("IlluminationCalibration")


# ---------------------------------------------------------------- geometry and fits (host)


def hann_window(shape):
    """skimage.filters.window("hann", shape): the symmetric 1-D Hann window
    of length max(shape), linearly interpolated (zero outside) at each
    pixel's distance from the centre, distances in float32."""
    shape = tuple(int(s) for s in shape)
    m = max(shape)
    w = 0.5 - 0.5 * np.cos(2.0 * np.pi * np.arange(m, dtype=np.float64) / (m - 1)) if m > 1 else np.ones(1)
    center = m / 2 - 0.5
    dist = np.float32(0)
    for ax, s in enumerate(shape):
        g = np.arange(s, dtype=np.float32) * np.float32(m / s)
        g -= np.float32(center)
        dist = dist + (g * g).reshape((-1,) + (1,) * (len(shape) - 1 - ax))
    c = (np.sqrt(dist) + np.float32(center)).astype(np.float64)
    i0 = np.floor(c).astype(np.int64)
    t = c - i0
    def at(i):
        ok = (i >= 0) & (i < m)
        return np.where(ok, w[np.clip(i, 0, m - 1)], 0.0)
    return at(i0) * (1.0 - t) + at(i0 + 1) * t


def gaussian_half_weights(sigma, truncate=4.0):
    """Radius and weights [centre, 1, ..., radius] of scipy.ndimage's 1-D
    Gaussian kernel, computed with the same NumPy expressions."""
    radius = int(truncate * float(sigma) + 0.5)
    x = np.arange(-radius, radius + 1)
    phi = np.exp(-0.5 / (sigma * sigma) * x**2)
    phi = phi / phi.sum()
    return radius, np.ascontiguousarray(phi[radius:], dtype=np.float64)


def kmeans2_labels(points, iterations=300):
    pts = np.asarray(points, dtype=np.float64)
    c = pts[[int(np.argmin(pts[:, -1])), int(np.argmax(pts[:, -1]))]].copy()
    labels = np.zeros(len(pts), dtype=int)
    for it in range(iterations):
        new = np.argmin(((pts[:, None, :] - c[None]) ** 2).sum(-1), axis=1)
        for j in range(2):
            if np.any(new == j):
                c[j] = pts[new == j].mean(0)
        if it > 0 and np.array_equal(new, labels):
            break
        labels = new
    return labels


def matrix_transform(coords, matrix):
    """Homogeneous 2-D transform of (n, 2) coordinates."""
    coords = np.asarray(coords, dtype=np.float64)
    src = np.column_stack([coords[:, 0], coords[:, 1], np.ones(len(coords))])
    dst = src @ np.asarray(matrix).T
    dst[dst[:, 2] == 0, 2] = np.finfo(float).eps
    return dst[:, :2] / dst[:, 2:3]


def _umeyama(src, dst, estimate_scale):
    # Umeyama (1991): least-squares rotation, scale and translation
    src = np.asarray(src, dtype=np.float64)
    dst = np.asarray(dst, dtype=np.float64)
    n, dim = src.shape
    sm, dm = src.mean(0), dst.mean(0)
    sd, dd = src - sm, dst - dm
    A = dd.T @ sd / n
    d = np.ones(dim)
    if np.linalg.det(A) < 0:
        d[dim - 1] = -1
    T = np.eye(dim + 1)
    U, S, Vt = np.linalg.svd(A)
    rank = np.linalg.matrix_rank(A)
    if rank == 0:
        return np.full((dim + 1, dim + 1), np.nan)
    if rank == dim - 1:
        if np.linalg.det(U) * np.linalg.det(Vt) > 0:
            T[:dim, :dim] = U @ Vt
        else:
            s = d[dim - 1]
            d[dim - 1] = -1
            T[:dim, :dim] = U @ np.diag(d) @ Vt
            d[dim - 1] = s
    else:
        T[:dim, :dim] = U @ np.diag(d) @ Vt
    scale = 1.0 / sd.var(0).sum() * (S @ d) if estimate_scale else 1.0
    T[:dim, dim] = dm - scale * (T[:dim, :dim] @ sm.T)
    T[:dim, :dim] *= scale
    return T


class _Transform:
    def __init__(self, matrix=None, translation=None):
        self.params = np.eye(3) if matrix is None else np.asarray(matrix, dtype=np.float64).copy()
        if translation is not None:
            self.params[0:2, 2] = translation

    @property
    def translation(self):
        return self.params[0:2, 2]

    def __call__(self, coords):
        return matrix_transform(coords, self.params)

    def residuals(self, src, dst):
        return np.sqrt(np.sum((self(src) - dst) ** 2, axis=1))


class EuclideanTransform(_Transform):
    def estimate(self, src, dst):
        self.params = _umeyama(src, dst, False)
        return bool(np.all(np.isfinite(self.params)))


class SimilarityTransform(_Transform):
    def estimate(self, src, dst):
        self.params = _umeyama(src, dst, True)
        return bool(np.all(np.isfinite(self.params)))


class AffineTransform(_Transform):
    def estimate(self, src, dst):
        X = np.column_stack([np.asarray(src, dtype=np.float64), np.ones(len(src))])
        sol, *_ = np.linalg.lstsq(X, np.asarray(dst, dtype=np.float64), rcond=None)
        self.params = np.eye(3)
        self.params[:2, :] = sol.T
        return bool(np.all(np.isfinite(self.params)))


def ransac(data, model_class, min_samples, residual_threshold, max_trials=100, stop_probability=1.0, seed=0):
    """RANSAC (Fischler & Bolles 1981) with scikit-image's stopping rule and
    a final fit on the best inlier set; fixed-seed draws."""
    src, dst = (np.asarray(d) for d in data)
    n = len(src)
    rng = np.random.default_rng(seed)
    eps = np.finfo(float).eps
    best_n, best_sum, best = 0, np.inf, None
    trials = 0
    while trials < max_trials:
        trials += 1
        idx = rng.choice(n, min_samples, replace=False)
        model = model_class()
        if not model.estimate(src[idx], dst[idx]):
            continue
        res = np.abs(model.residuals(src, dst))
        inl = res < residual_threshold
        rsum = res.dot(res)
        cnt = int(np.count_nonzero(inl))
        if cnt > best_n or (cnt == best_n and rsum < best_sum):
            best_n, best_sum, best = cnt, rsum, inl
            denom = max(eps, 1 - (best_n / n) ** min_samples)
            if trials >= np.ceil(np.log(max(eps, 1 - stop_probability)) / np.log(denom)):
                break
    if best is None or not np.any(best):
        return None, None
    model = model_class()
    model.estimate(src[best], dst[best])
    return model, best


# ---------------------------------------------------------------- device calls


_FRAUNHOFER, _INVERSE = 0, 1  # enum ptyg_propagator / ptyg_direction


def _ptr(t):
    return C.c_void_p(t.data_ptr())


def _host_ptr(a):
    return a.ctypes.data_as(C.c_void_p)


class _Device:
    """libptyg's calibration calls on one CUDA device."""

    def __init__(self, device=None):
        import torch

        self.torch = torch
        self.device = torch.device("cuda", torch.cuda.current_device()) if device is None else torch.device(device)
        self.lib = _native.require(self.device.index if self.device.index is not None else 0)

    def stream(self):
        return C.c_void_p(self.torch.cuda.current_stream(self.device).cuda_stream)

    def take(self, arr, idx):
        """Rows ``idx`` of a device array, contiguous."""
        i = self.torch.as_tensor(np.asarray(idx, dtype=np.int64), device=self.device)
        return arr.index_select(0, i).contiguous()

    def to_host(self, arr):
        return arr.cpu().numpy()

    def upload(self, arr):
        return self.torch.from_numpy(np.ascontiguousarray(arr, dtype=np.float32)).to(self.device)

    def ifft2c(self, images):
        """Centred inverse transforms (complex64) of real device frames."""
        torch = self.torch
        n, N, _ = images.shape
        z = images.to(torch.complex64).contiguous()
        out = torch.empty_like(z)
        self.check(self.lib.ptyg_propagate(_FRAUNHOFER, _INVERSE, 0, N, n, _ptr(z), _ptr(out), None, None,
                                           self.stream()), "ptyg_propagate")
        return out

    def check(self, status, name):
        _native.check(status, name)

    def spectra(self, frames_host, window):
        torch = self.torch
        n, N, N2 = frames_host.shape
        if N != N2 or window.shape != (N, N):
            raise ValueError("frames must be square and the window their size")
        frames = torch.from_numpy(np.ascontiguousarray(frames_host, dtype=np.float32)).to(self.device)
        win = torch.from_numpy(np.ascontiguousarray(window, dtype=np.float64)).to(self.device)
        windowed = torch.empty_like(frames)
        sums = torch.empty(n, dtype=torch.float64, device=self.device)
        spectra = torch.empty((n, N, N), dtype=torch.complex64, device=self.device)
        ft = torch.empty_like(frames)
        norm = torch.empty((N, N), dtype=torch.float32, device=self.device)
        self.check(self.lib.ptyg_calib_spectra(n, N, _ptr(frames), _ptr(win), _ptr(windowed), _ptr(sums),
                                               _ptr(spectra), _ptr(ft), _ptr(norm), self.stream()),
                   "ptyg_calib_spectra")
        return windowed, sums, spectra, ft, norm

    def normalise(self, ft, norm, floor_value):
        n, N, _ = ft.shape
        self.check(self.lib.ptyg_calib_normalise(n, N, _ptr(ft), _ptr(norm), C.c_float(float(floor_value)),
                                                 self.stream()), "ptyg_calib_normalise")

    def gaussian(self, images, sigma, out=None):
        n, N, _ = images.shape
        out = images if out is None else out
        radius, w = gaussian_half_weights(sigma)
        self.check(self.lib.ptyg_calib_gaussian(n, N, radius, _host_ptr(w), _ptr(images), _ptr(out),
                                                self.stream()), "ptyg_calib_gaussian")
        return out

    def arcs(self, images, task_image, task_pos, task_keep, radii, sin_a, cos_a, search):
        """circleSearchArray (tasks, R, G, G) float32, on the host."""
        torch = self.torch
        N = images.shape[-1]
        T = len(task_image)
        G = 2 * search + 1
        out = torch.empty((T, len(radii), G, G), dtype=torch.float32, device=self.device)
        if T == 0:
            return out.cpu().numpy()
        if min(task_image) < 0 or max(task_image) >= images.shape[0]:
            raise ValueError("task image index outside the image stack")
        if len(radii) > 64 or len(sin_a) > 64:
            raise ValueError("at most 64 radii and 64 angles")
        ti = torch.as_tensor(np.asarray(task_image, dtype=np.int32), device=self.device)
        tp = torch.as_tensor(np.asarray(task_pos, dtype=np.float64).reshape(-1), device=self.device)
        tk = torch.as_tensor(np.asarray(task_keep, dtype=np.uint64).view(np.int64), device=self.device)
        radii = np.ascontiguousarray(radii, dtype=np.float64)
        sin_a = np.ascontiguousarray(sin_a, dtype=np.float64)
        cos_a = np.ascontiguousarray(cos_a, dtype=np.float64)
        self.check(self.lib.ptyg_calib_arcs(N, _ptr(images), T, _ptr(ti), _ptr(tp), _ptr(tk), len(radii),
                                            _host_ptr(radii), len(sin_a), _host_ptr(sin_a), _host_ptr(cos_a),
                                            int(search), _ptr(out), self.stream()), "ptyg_calib_arcs")
        return out.cpu().numpy()

    def rms(self, spectra, images, cand_led, cand_q, radius):
        torch = self.torch
        N = images.shape[-1]
        K = len(cand_led)
        out = torch.empty(K, dtype=torch.float64, device=self.device)
        if K == 0:
            return np.zeros(0)
        if min(cand_led) < 0 or max(cand_led) >= min(spectra.shape[0], images.shape[0]):
            raise ValueError("candidate frame index outside the frame stack")
        if spectra.dtype != torch.complex64 or images.dtype != torch.float32:
            raise ValueError("spectra must be complex64 and images float32")
        cl = torch.as_tensor(np.asarray(cand_led, dtype=np.int32), device=self.device)
        cq = torch.as_tensor(np.asarray(cand_q, dtype=np.int32).reshape(-1), device=self.device)
        self.check(self.lib.ptyg_calib_rms(N, _ptr(spectra), _ptr(images), K, _ptr(cl), _ptr(cq),
                                           C.c_double(float(radius)), _ptr(out), self.stream()), "ptyg_calib_rms")
        return out.cpu().numpy()


# ---------------------------------------------------------------- the calibration


class IlluminationCalibration:
    def __init__(self, reconstructor, experimentalData):
        """CalibrationFPM.py:34-65."""
        self.reconstructor = reconstructor
        self.experimentalData = experimentalData
        self.searchGridSize = round(int(reconstructor.Np * 0.1))
        self.gaussSigma = 3
        self.plot = False
        self.calibrateRadius = False
        self.brightfieldIndices = None
        self.fit_mode = "SimilarityTransform"
        self.dxp = reconstructor.dxp
        self.No = reconstructor.No
        self.Np = reconstructor.Np
        self.wavelength = reconstructor.wavelength
        self.img_size = reconstructor.Np
        self.apertRadiusPixel = self.dxp * self.img_size * self.reconstructor.NA / self.wavelength
        self.apertRadiusPixel_init = self.apertRadiusPixel
        lens_range = np.linspace(-self.img_size / 2, self.img_size / 2, self.img_size)
        xlens, ylens = np.meshgrid(lens_range, lens_range)
        self.CTF = np.abs(np.sqrt(xlens**2 + ylens**2) <= self.apertRadiusPixel)
        self.OTF = np.abs(np.sqrt(xlens**2 + ylens**2) <= 2 * self.apertRadiusPixel)
        self._dev = None

    # -------------------------------------------------------------- pieces
    def _device(self):
        if self._dev is None:
            self._dev = _Device()
        return self._dev

    def initialize_error_search_space(self):
        """CalibrationFPM.py:67-77."""
        self.angleRange_x_init = np.sin(np.mgrid[0:360:10] / 180.0 * np.pi)
        self.angleRange_y_init = np.cos(np.mgrid[0:360:10] / 180.0 * np.pi)
        self.gridSearch_x_init = np.mgrid[-self.searchGridSize:self.searchGridSize + 1]
        self.gridSearch_y_init = np.mgrid[-self.searchGridSize:self.searchGridSize + 1]
        self.x_range = len(self.gridSearch_x_init)
        self.y_range = len(self.gridSearch_y_init)

    def _fourier(self, ptychogram, smooth=True):
        """convertToFourierSpace on the device: (windowed frames, frame sums,
        inverse transforms of the windowed frames, normalised Fourier
        magnitudes, Gaussian-smoothed unless ``smooth`` is False)."""
        dev = self._device()
        if self.img_size not in (32, 64, 128, 256) or ptychogram.shape[-1] != self.img_size:
            raise NotImplementedError("the calibration kernels take frames of 32, 64, 128 or 256 pixels")
        windowed, sums, spectra, ft, norm = dev.spectra(ptychogram, hann_window(ptychogram[0].shape))
        normalization = dev.to_host(norm)
        mean_outside_support = np.mean(normalization[self.OTF == 0])
        dev.normalise(ft, norm, np.float32(2 * mean_outside_support))
        if smooth:
            dev.gaussian(ft, self.gaussSigma)
        return windowed, dev.to_host(sums), spectra, ft

    def convertToFourierSpace(self, ptychogram):
        """CalibrationFPM.py:113-147: windows ``ptychogram`` in place and
        returns the contrast-enhanced |ifft2c| of every frame."""
        windowed, _, _, ft = self._fourier(ptychogram)
        dev = self._device()
        ptychogram[...] = dev.to_host(windowed)
        return dev.to_host(ft)

    def findBrightfielIndices(self, ptychogram=None, frame_sums=None):
        """CalibrationFPM.py:79-111: two-cluster split on (frame index,
        frame intensity); the cluster of larger mean intensity is brightfield."""
        if frame_sums is None:
            frame_sums = np.sum(np.asarray(ptychogram, dtype=np.float64), (1, 2))
        intensities = np.asarray(frame_sums, dtype=np.float64)
        labels = kmeans2_labels(np.array([np.arange(len(intensities)), intensities]).T)
        c1, c2 = labels == 0, labels == 1
        m1 = intensities[c1].sum() / max(1, c1.sum())
        m2 = intensities[c2].sum() / max(1, c2.sum())
        return c1 if m1 > m2 else c2

    def _keep_angles(self, position, radii):
        """The angles whose circle points stay inside (1, N - 1) for every
        radius and grid shift (CalibrationFPM.py:232-241).  float32 rounding
        is monotone, so the extreme grid shifts decide."""
        g = np.array([-self.searchGridSize, self.searchGridSize]).reshape(1, 2, 1)
        R = np.asarray(radii, dtype=np.float64).reshape(-1, 1, 1)
        ax = self.angleRange_x_init.reshape(1, 1, -1)
        ay = self.angleRange_y_init.reshape(1, 1, -1)
        xx = np.single(R * ax + self.img_size / 2.0 + position[0] + g)
        yy = np.single(R * ay + self.img_size / 2.0 + position[1] + g)
        ok = (yy > 1) & (xx > 1) & (xx < self.img_size - 1) & (yy < self.img_size - 1)
        keep = np.all(ok, axis=(0, 1))
        return int(np.sum(keep.astype(np.uint64) << np.arange(keep.size, dtype=np.uint64)))

    def _circle_search(self, images, image_index, positions, radii):
        """circleSearchArray per task: (tasks, R, G, G) float32."""
        dev = self._device()
        keep = [self._keep_angles(p, radii) for p in positions]
        return dev.arcs(images, image_index, np.asarray(positions, dtype=np.float64), keep, radii,
                        self.angleRange_x_init, self.angleRange_y_init, self.searchGridSize)

    def generateCircularArcsVectorized(self, initialPositions):
        """CalibrationFPM.py:149-288 (host): the (R, G, G, P, 2) sample
        coordinates for the current ``radiusScanRangeInit``."""
        g = self.gridSearch_x_init
        gy, gx = np.meshgrid(g, g)
        gx = gx.reshape(1, len(g), len(g), 1)
        gy = gy.reshape(1, len(g), len(g), 1)
        R = np.asarray(self.radiusScanRangeInit).reshape(-1, 1, 1, 1)
        ax = self.angleRange_x_init.reshape(1, 1, 1, -1)
        ay = self.angleRange_y_init.reshape(1, 1, 1, -1)
        keep = self._keep_angles(initialPositions, self.radiusScanRangeInit)
        sel = np.array([(keep >> k) & 1 for k in range(ax.size)], dtype=bool)
        arcs = np.zeros([R.shape[0], len(g), len(g), int(sel.sum()), 2])
        arcs[..., 0] = np.single(R * ax[..., sel] + self.img_size / 2.0 + initialPositions[0] + gx)
        arcs[..., 1] = np.single(R * ay[..., sel] + self.img_size / 2.0 + initialPositions[1] + gy)
        return arcs

    def computePositionErrorCandidates(self, circleSearchArray):
        """CalibrationFPM.py:360-419."""
        arc_dx1 = np.diff(circleSearchArray, n=1, axis=0)
        rad_dx_idx = np.argwhere(np.max(arc_dx1) == arc_dx1)[0][0]
        search_grid_dx = np.squeeze(arc_dx1[rad_dx_idx, :, :])
        search_grid_dx = search_grid_dx >= np.max(search_grid_dx) - 0.1 * np.std(search_grid_dx)
        return np.argwhere(search_grid_dx > 0)

    def _decide(self, candidates, rms):
        """CalibrationFPM.py:340-358: best candidate and the edge flag."""
        k = int(np.argmin(rms))
        ex = self.gridSearch_x_init[int(candidates[k, 0])]
        ey = self.gridSearch_y_init[int(candidates[k, 1])]
        b = (0, len(self.gridSearch_x_init) - 1)
        edge = candidates[k, 0] in b or candidates[k, 1] in b
        return ex, ey, edge

    def calculateRMSE(self, image, error_candidates, position):
        """CalibrationFPM.py:290-358 for one frame (host array), on the
        device; returns (error x, error y, on the grid's edge)."""
        dev = self._device()
        img = dev.upload(np.asarray(image)[None])
        q = np.stack([position[0] + self.gridSearch_x_init[error_candidates[:, 0]],
                      position[1] + self.gridSearch_y_init[error_candidates[:, 1]]], 1)
        rms = dev.rms(dev.ifft2c(img), img, np.zeros(len(q), dtype=np.int32), q, self.apertRadiusPixel)
        return self._decide(error_candidates, rms)

    # -------------------------------------------------------------- the two searches
    def findCalibratedRadius(self, ptychogram, FT_ptychogram, initialPositions):
        """CalibrationFPM.py:421-536; ``FT_ptychogram``, the brightfield
        frames' Fourier images, as a host array or a device tensor."""
        self.initialize_error_search_space()
        self.radiuSearchBounds = 5
        self.radiusSearchStep = 0.5
        self.radiusSearchRange = np.mgrid[self.radiuSearchBounds:-self.radiuSearchBounds
                                          - self.radiusSearchStep:-self.radiusSearchStep]
        tolerance = [self.radiusSearchStep * 1.1, self.radiusSearchStep * 0.9]
        self.apertRadiusPixel_init = self.apertRadiusPixel
        dev = self._device()
        if isinstance(FT_ptychogram, np.ndarray):  # PtyLab's callers pass host arrays
            FT_ptychogram = dev.upload(FT_ptychogram)
        initialPositions = np.asarray(initialPositions)
        nimg = FT_ptychogram.shape[0]
        converged = False
        check_done = False
        radii_array = [self.apertRadiusPixel]
        itr = 0
        while not converged:
            logger.info("Radius %spx, iteration %s", self.apertRadiusPixel, itr)
            itr += 1
            radiiIdxForEachImg = np.zeros(nimg)
            self.radiusScanRangeInit = self.radiusSearchRange + self.apertRadiusPixel
            idx_range = np.arange(nimg)
            if nimg > 20:
                np.random.shuffle(idx_range)
                idx_range = idx_range[:20]
            blurred = dev.gaussian(dev.take(FT_ptychogram, idx_range), self.gaussSigma)
            cs = self._circle_search(blurred, np.arange(len(idx_range)), initialPositions[idx_range],
                                     self.radiusScanRangeInit)
            for t, idx in enumerate(idx_range):
                arc_dx1 = np.gradient(cs[t], axis=0)
                radiiIdxForEachImg[idx] = np.argwhere(np.max(arc_dx1) == arc_dx1)[0][0]
            radius_index = int(np.median(radiiIdxForEachImg))
            self.apertRadiusPixel = self.radiusScanRangeInit[radius_index]
            radii_array.append(self.apertRadiusPixel)
            if not check_done:
                if abs(radii_array[-1] - radii_array[-2]) <= tolerance[0]:
                    check_done = True
            else:
                mean_rad = np.mean(radii_array[-2:])
                if abs(mean_rad - radii_array[-1]) <= tolerance[1]:
                    self.apertRadiusPixel = mean_rad
                    converged = True
                else:
                    check_done = False
            if (itr >= 20 and not check_done) or self.apertRadiusPixel <= 0:
                self.apertRadiusPixel = self.apertRadiusPixel_init
                converged = True
        return self.apertRadiusPixel_init, self.apertRadiusPixel

    def findPositionCalibrationMatrix(self, ptychogram, FT_ptychogram, initialPositions, spectra=None):
        """CalibrationFPM.py:538-665 with every LED searched at once:
        ``ptychogram`` (windowed frames) and ``FT_ptychogram`` of the
        brightfield frames as host arrays or device tensors; ``spectra``
        (their inverse transforms) is computed when not given."""
        self.initialize_error_search_space()
        dev = self._device()
        if isinstance(ptychogram, np.ndarray):  # PtyLab's callers pass host arrays
            ptychogram = dev.upload(ptychogram)
        if isinstance(FT_ptychogram, np.ndarray):
            FT_ptychogram = dev.upload(FT_ptychogram)
        initialPositions = np.asarray(initialPositions)
        nimg = FT_ptychogram.shape[0]
        calibrated = np.array(initialPositions, copy=True)
        failed = []
        self.radiusSearchStep = 0.5
        self.radiusSearchRange = np.mgrid[max(self.gaussSigma + 2 * self.radiusSearchStep,
                                              3 * self.radiusSearchStep):-self.radiusSearchStep:
                                          -self.radiusSearchStep]
        self.radiusScanRangeInit = self.radiusSearchRange + self.apertRadiusPixel
        if spectra is None:
            spectra = dev.ifft2c(ptychogram)
        repeats = np.zeros(nimg, dtype=int)
        active = list(range(nimg))
        self.rounds = 0
        while active:
            self.rounds += 1
            cs = self._circle_search(FT_ptychogram, active, calibrated[active], self.radiusScanRangeInit)
            cand_of, led_of, q_of = {}, [], []
            for t, idx in enumerate(active):
                try:
                    cand = self.computePositionErrorCandidates(cs[t])
                except Exception:  # noqa: BLE001 - the reference records the frame as failed
                    failed.append(idx)
                    continue
                cand_of[idx] = (cand, len(led_of))
                for c in cand:
                    led_of.append(idx)
                    q_of.append((calibrated[idx, 0] + self.gridSearch_x_init[int(c[0])],
                                 calibrated[idx, 1] + self.gridSearch_y_init[int(c[1])]))
            rms = dev.rms(spectra, ptychogram, led_of, q_of, self.apertRadiusPixel)
            still = []
            for idx, (cand, start) in cand_of.items():
                ex, ey, edge = self._decide(cand, rms[start:start + len(cand)])
                calibrated[idx, 0] = calibrated[idx, 0] + ex
                calibrated[idx, 1] = calibrated[idx, 1] + ey
                if edge and repeats[idx] < 5:
                    repeats[idx] += 1
                    still.append(idx)
            active = still
        failed = sorted(failed)
        self.calibrated_positions = calibrated
        self.failed_position_calib = failed
        if len(failed) != nimg:
            src = np.delete(initialPositions, failed, axis=0)
            dst = np.delete(calibrated, failed, axis=0)
            calibMatrix, updatedPositions = self.fitCoordinates(src, dst, self.fit_mode)
            updatedPositions = matrix_transform(initialPositions, calibMatrix.params)
        else:
            calibMatrix = SimilarityTransform(np.eye(3))
            updatedPositions = initialPositions
        return calibMatrix, updatedPositions

    def plotCalibration(self, FT_ptychogram, initialPositions, calibrated_positions):
        """CalibrationFPM.py:667-743 draws the fitted circles with matplotlib;
        no plotting is available here."""
        raise NotImplementedError("plotting the calibration is not available")

    def fitCoordinates(self, src, dst, mode):
        """CalibrationFPM.py:745-789."""
        if mode in ("Translation", "EuclideanTransform"):
            cls = EuclideanTransform
        elif mode == "SimilarityTransform":
            cls = SimilarityTransform
        elif mode == "AffineTransform":
            cls = AffineTransform
        else:
            cls = EuclideanTransform
            logger.warning("Required fit mode not found, using EuclideanTransform")
        resThresh = np.median(np.abs(dst - src))
        matrix, inliers = ransac((src, dst), cls, min_samples=2, residual_threshold=resThresh, max_trials=10000)
        if matrix is None:
            raise RuntimeError("no inliers: the calibrated positions fit no transform")
        if mode == "Translation":
            matrix = cls(translation=matrix.translation)
        return matrix, matrix_transform(src, matrix.params)

    def updatePositions(self):
        """CalibrationFPM.py:791-828: the calibration in encoder units."""
        conv = -(1 / self.reconstructor.wavelength) * self.reconstructor.dxo * self.reconstructor.Np
        z = self.reconstructor.zled
        P = self.calibMatrix.params.copy()
        E = self.calibMatrix.params.copy()
        E[0:2, 2] = np.sign(conv) * P[0:2, 2] * z / (np.sqrt(conv**2 - P[0, 2] ** 2 - P[1, 2] ** 2))
        self.experimentalData.encoder = matrix_transform(self.experimentalData.encoder, E)
        self.reconstructor.positions0 = self.reconstructor.positions.copy()

    def runCalibration(self):
        """CalibrationFPM.py:830-919."""
        if self.plot:
            raise NotImplementedError("plotting the calibration is not available")
        # the windowed frames go to a new device buffer, so the data's frames
        # are read as they are (the reference deep-copies them to window in place)
        ptychogram = np.asarray(self.experimentalData.ptychogram, dtype=np.float32)
        self.initialPositions = np.array(self.reconstructor.positions, copy=True)
        self.initialPositions = self.initialPositions - self.reconstructor.No // 2 + self.reconstructor.Np // 2
        self.initialize_error_search_space()
        # the smoothing is per frame and only the brightfield frames are
        # searched, so only they are smoothed (the reference smooths all)
        windowed, sums, spectra, ft = self._fourier(ptychogram, smooth=False)
        if not hasattr(self.brightfieldIndices, "__len__"):
            self.brightfieldIndices = self.findBrightfielIndices(frame_sums=sums)
        bf = np.asarray(self.brightfieldIndices)
        bf_idx = np.flatnonzero(bf) if bf.dtype == bool else bf
        dev = self._device()
        ft_bf = dev.gaussian(dev.take(ft, bf_idx), self.gaussSigma)
        if self.calibrateRadius:
            oldRadius, newRadius = self.findCalibratedRadius(None, ft_bf, self.initialPositions[bf])
            logger.info("Initial radius was %spx, calibrated radius is %spx", np.round(oldRadius, 2),
                        np.round(newRadius, 2))
            self.reconstructor.NA = np.round(newRadius / self.dxp * self.wavelength / self.img_size, 3)
            self.apertRadiusPixel = newRadius
        else:
            self.reconstructor.NA = self.apertRadiusPixel / self.dxp * self.wavelength / self.img_size
        self.calibMatrix, _ = self.findPositionCalibrationMatrix(
            dev.take(windowed, bf_idx), ft_bf, self.initialPositions[bf, :], spectra=dev.take(spectra, bf_idx))
        positionsFitted = matrix_transform(self.initialPositions, self.calibMatrix.params)
        self.reconstructor.entrancePupilDiameter = self.apertRadiusPixel * self.dxp * 2
        self.positionsFitted = positionsFitted.astype(int)
        self.updatePositions()
        return self.calibMatrix
