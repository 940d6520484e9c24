"""CPU restatement of PtyLab's FPM illumination calibration
(PtyLab/Reconstruction/CalibrationFPM.py:33-919).

TEST INFRASTRUCTURE ONLY: the checker for ``ptylab_gb300.CalibrationFPM``.
Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU legs may
import it; the package never does.

The reference calls five third-party routines that are not installed here
(scikit-image) or not on the GPU host (scikit-learn).  They are restated from
their published definitions, and ``tests/golden/make_calib_golden.py`` runs
the reference's own ``IlluminationCalibration`` with these restatements in
place of scikit-image (and scikit-learn's real KMeans), so the goldens pin
the reference's logic on top of them:

* ``skimage.filters.window("hann", shape)``: a radially symmetric window,
  the symmetric 1-D Hann window of length max(shape) sampled by linear
  interpolation (zero outside) at each pixel's distance from the centre;
* ``skimage.filters.gaussian(img, sigma)``:
  ``scipy.ndimage.gaussian_filter(img, sigma, mode="nearest", truncate=4)``
  into an array of the image's floating type;
* ``sklearn.cluster.KMeans(n_clusters=2)``: Lloyd iterations from the
  lowest- and highest-intensity frames (the labels' order is irrelevant: the
  reference picks the cluster with the larger mean);
* ``skimage.measure.ransac`` (Fischler & Bolles 1981) with its stopping rule
  and a final fit on the best inlier set; ``EuclideanTransform`` /
  ``SimilarityTransform`` by Umeyama's least-squares estimate (1991),
  ``AffineTransform`` by linear least squares; ``matrix_transform`` in
  homogeneous coordinates.
"""

from __future__ import annotations

import math

import numpy as np
from scipy.ndimage import gaussian_filter, map_coordinates


def ifft2c(x):
    """PtyLab/utils/utils.py:31-49 (centred, unitary)."""
    return np.fft.fftshift(np.fft.ifft2(np.fft.ifftshift(x, axes=(-2, -1)), norm="ortho"), axes=(-2, -1))


# ---------------------------------------------------------------- restated third-party routines


def hann_window(shape):
    """Radially symmetric Hann window of ``shape`` (float64)."""
    shape = tuple(int(s) for s in shape)
    m = max(shape)
    k = np.arange(m, dtype=np.float64)
    w = 0.5 - 0.5 * np.cos(2.0 * np.pi * k / (m - 1)) if m > 1 else np.ones(1)
    center = m / 2 - 0.5
    dist = np.float32(0)
    for ax, s in enumerate(shape):
        g = np.arange(s, dtype=np.float32) * np.float32(m / s)
        g -= np.float32(center)
        g = g.reshape((-1,) + (1,) * (len(shape) - 1 - ax))
        dist = dist + g * g
    coord = (np.sqrt(dist) + np.float32(center)).astype(np.float32)
    return map_coordinates(w[:, None], np.stack([coord, np.zeros_like(coord)]), order=1, mode="constant", cval=0.0)


def gaussian(img, sigma):
    """skimage.filters.gaussian for a float image."""
    img = np.asarray(img)
    out = np.empty_like(img, dtype=img.dtype if img.dtype.kind == "f" else np.float64)
    gaussian_filter(img, sigma, output=out, mode="nearest", truncate=4.0)
    return out


def kmeans2_labels(points, iterations=300):
    """Two-cluster Lloyd iterations on ``points`` (n, d), seeded with the
    points of lowest and highest last coordinate (the frame intensity)."""
    pts = np.asarray(points, dtype=np.float64)
    c = pts[[int(np.argmin(pts[:, -1])), int(np.argmax(pts[:, -1]))]].copy()
    labels = np.zeros(len(pts), dtype=int)
    for _ in range(iterations):
        d = ((pts[:, None, :] - c[None]) ** 2).sum(-1)
        new = np.argmin(d, axis=1)
        for j in range(2):
            if np.any(new == j):
                c[j] = pts[new == j].mean(0)
        if np.array_equal(new, labels) and _ > 0:
            break
        labels = new
    return labels


def matrix_transform(coords, matrix):
    coords = np.asarray(coords, dtype=np.float64)
    src = np.column_stack([coords[:, 0], coords[:, 1], np.ones(len(coords))])
    dst = src @ np.asarray(matrix).T
    dst[dst[:, 2] == 0, 2] = np.finfo(float).eps
    return dst[:, :2] / dst[:, 2:3]


def umeyama(src, dst, estimate_scale):
    """Least-squares rotation (+ scale) and translation taking src to dst."""
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
        self.params = umeyama(src, dst, False)
        return bool(np.all(np.isfinite(self.params)))


class SimilarityTransform(_Transform):
    def estimate(self, src, dst):
        self.params = umeyama(src, dst, True)
        return bool(np.all(np.isfinite(self.params)))


class AffineTransform(_Transform):
    def estimate(self, src, dst):
        src = np.asarray(src, dtype=np.float64)
        dst = np.asarray(dst, dtype=np.float64)
        X = np.column_stack([src, np.ones(len(src))])
        sol, *_ = np.linalg.lstsq(X, dst, rcond=None)
        self.params = np.eye(3)
        self.params[:2, :] = sol.T
        return bool(np.all(np.isfinite(self.params)))


TRANSFORMS = {"EuclideanTransform": EuclideanTransform, "SimilarityTransform": SimilarityTransform,
              "AffineTransform": AffineTransform}


def _dynamic_max_trials(n_inliers, n_samples, min_samples, probability):
    if n_inliers == 0:
        return np.inf
    eps = np.finfo(float).eps
    nom = max(eps, 1 - probability)
    denom = max(eps, 1 - (n_inliers / n_samples) ** min_samples)
    return np.ceil(np.log(nom) / np.log(denom))


def ransac(data, model_class, min_samples, residual_threshold, max_trials=100, stop_probability=1.0, seed=0):
    """RANSAC with the stopping rule of skimage.measure.ransac; the model is
    refitted on the best inlier set.  Returns (model or None, inliers)."""
    src, dst = (np.asarray(d) for d in data)
    n = len(src)
    rng = np.random.default_rng(seed)
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
            if trials >= _dynamic_max_trials(best_n, n, min_samples, stop_probability):
                break
    if best is None or not np.any(best):
        return None, None
    model = model_class()
    model.estimate(src[best], dst[best])
    return model, best


# ---------------------------------------------------------------- the calibration


class CalibrationOracle:
    """The reference's IlluminationCalibration state and steps, NumPy/SciPy."""

    def __init__(self, Np, No, dxp, wavelength, NA, searchGridSize=None, gaussSigma=3,
                 calibrateRadius=False, fit_mode="SimilarityTransform", brightfieldIndices=None):
        # CalibrationFPM.py:34-65
        self.searchGridSize = round(int(Np * 0.1)) if searchGridSize is None else searchGridSize
        self.gaussSigma = gaussSigma
        self.calibrateRadius = calibrateRadius
        self.brightfieldIndices = brightfieldIndices
        self.fit_mode = fit_mode
        self.dxp, self.No, self.Np, self.wavelength = dxp, No, Np, wavelength
        self.img_size = Np
        self.apertRadiusPixel = dxp * Np * NA / wavelength
        self.apertRadiusPixel_init = self.apertRadiusPixel
        r = np.linspace(-Np / 2, Np / 2, Np)
        xl, yl = np.meshgrid(r, r)
        self.OTF = np.abs(np.sqrt(xl**2 + yl**2) <= 2 * self.apertRadiusPixel)
        self.NA = NA
        self.initialize_error_search_space()

    def initialize_error_search_space(self):
        """CalibrationFPM.py:67-77."""
        self.angleRange_x_init = np.sin(np.mgrid[0:360:10] / 180.0 * np.pi)
        self.angleRange_y_init = np.cos(np.mgrid[0:360:10] / 180.0 * np.pi)
        self.gridSearch_init = np.mgrid[-self.searchGridSize:self.searchGridSize + 1]

    def convertToFourierSpace(self, ptychogram):
        """CalibrationFPM.py:113-147: windows ``ptychogram`` in place."""
        ptychogram *= hann_window(ptychogram[0].shape)[None, ...]
        ft = np.abs(ifft2c(ptychogram))
        norm = np.mean(ft, 0)
        mean_outside = np.mean(norm[self.OTF == 0])
        norm = np.maximum(norm, 2 * mean_outside)
        ft = np.abs(ft / norm)
        for i in range(ft.shape[0]):
            ft[i] = gaussian(ft[i], self.gaussSigma)
        return ft

    @staticmethod
    def findBrightfielIndices(ptychogram):
        """CalibrationFPM.py:79-111."""
        intensities = np.sum(ptychogram, (1, 2))
        labels = kmeans2_labels(np.array([np.arange(ptychogram.shape[0]), intensities]).T)
        c1, c2 = labels == 0, labels == 1
        return c1 if np.mean(ptychogram[c1]) > np.mean(ptychogram[c2]) else c2

    def circular_arcs(self, position, radii):
        """CalibrationFPM.py:149-288: sample coordinates (R, G, G, P, 2) of the
        circles of every radius and grid shift, keeping the angles whose
        points stay inside (1, N-1) for all of them."""
        g = self.gridSearch_init
        gy, gx = np.meshgrid(g, g)
        gx = gx.reshape(1, len(g), len(g), 1)
        gy = gy.reshape(1, len(g), len(g), 1)
        R = np.asarray(radii).reshape(-1, 1, 1, 1)
        ax = self.angleRange_x_init.reshape(1, 1, 1, -1)
        ay = self.angleRange_y_init.reshape(1, 1, 1, -1)
        xx = np.single(R * ax + self.img_size / 2.0 + position[0] + gx).reshape(-1, ax.size)
        yy = np.single(R * ay + self.img_size / 2.0 + position[1] + gy).reshape(-1, ay.size)
        keep = np.all((yy > 1) * (xx > 1) * (xx < self.img_size - 1) * (yy < self.img_size - 1), 0)
        arcs = np.zeros([len(radii), len(g), len(g), int(np.count_nonzero(keep)), 2])
        arcs[..., 0] = np.single(R * ax[..., keep] + self.img_size / 2.0 + position[0] + gx)
        arcs[..., 1] = np.single(R * ay[..., keep] + self.img_size / 2.0 + position[1] + gy)
        return arcs

    def circle_search(self, image, position, radii):
        arcs = self.circular_arcs(position, radii)
        coords = np.array([arcs[..., 0].ravel(), arcs[..., 1].ravel()])
        vals = map_coordinates(image, coords, order=1, prefilter=False)
        return np.mean(np.reshape(vals, arcs.shape[:-1]), 3)

    @staticmethod
    def computePositionErrorCandidates(circleSearchArray):
        """CalibrationFPM.py:360-419."""
        d1 = np.diff(circleSearchArray, n=1, axis=0)
        i1 = np.argwhere(np.max(d1) == d1)[0][0]
        grid = np.squeeze(d1[i1, :, :])
        grid = grid >= np.max(grid) - 0.1 * np.std(grid)
        return np.argwhere(grid > 0)

    def calculateRMSE(self, image, candidates, position):
        """CalibrationFPM.py:290-358."""
        n = self.img_size
        xx, yy = np.mgrid[0:n, 0:n]
        F = ifft2c(image)
        rms, xs, ys = [], [], []
        for c in candidates:
            ex = self.gridSearch_init[int(c[0])]
            ey = self.gridSearch_init[int(c[1])]
            pupil = np.zeros(F.shape)
            pupil[((xx - n / 2.0 + (position[0] + ex)) ** 2 + (yy - n / 2.0 + (position[1] + ey)) ** 2)
                  <= self.apertRadiusPixel**2] = 1
            est = np.abs(ifft2c(pupil * F))
            rms.append(np.sqrt(np.mean((image - est) ** 2)))
            xs.append(ex)
            ys.append(ey)
        k = int(np.argmin(rms))
        b = (0, len(self.gridSearch_init) - 1)
        edge = candidates[k, 0] in b or candidates[k, 1] in b
        return xs[k], ys[k], edge, np.asarray(rms)

    def findCalibratedRadius(self, FT, positions):
        """CalibrationFPM.py:421-536 (global NumPy RNG for the 20-image subset)."""
        bounds, step = 5, 0.5
        search = np.mgrid[bounds:-bounds - step:-step]
        tol = [step * 1.1, step * 0.9]
        self.apertRadiusPixel_init = self.apertRadiusPixel
        converged, check_done = False, False
        radii = [self.apertRadiusPixel]
        itr = 0
        while not converged:
            itr += 1
            best = np.zeros(FT.shape[0])
            scan = search + self.apertRadiusPixel
            idx_range = np.arange(FT.shape[0])
            if FT.shape[0] > 20:
                np.random.shuffle(idx_range)
                idx_range = idx_range[:20]
            for idx in idx_range:
                image = gaussian(FT[idx], self.gaussSigma)
                cs = self.circle_search(image, positions[idx, :], scan)
                d1 = np.gradient(cs, axis=0)
                best[idx] = np.argwhere(np.max(d1) == d1)[0][0]
            self.apertRadiusPixel = scan[int(np.median(best))]
            radii.append(self.apertRadiusPixel)
            if not check_done:
                if abs(radii[-1] - radii[-2]) <= tol[0]:
                    check_done = True
            else:
                mean_rad = np.mean(radii[-2:])
                if abs(mean_rad - radii[-1]) <= tol[1]:
                    self.apertRadiusPixel = mean_rad
                    converged = True
                else:
                    check_done = False
            if (itr >= 20 and not check_done) or self.apertRadiusPixel <= 0:
                self.apertRadiusPixel = self.apertRadiusPixel_init
                converged = True
        return self.apertRadiusPixel_init, self.apertRadiusPixel

    def findPositionCalibrationMatrix(self, frames, FT, positions):
        """CalibrationFPM.py:538-665."""
        calibrated = positions.copy()
        failed = []
        step = 0.5
        scan = np.mgrid[max(self.gaussSigma + 2 * step, 3 * step):-step:-step] + self.apertRadiusPixel
        self.rounds = np.zeros(FT.shape[0], dtype=int)
        for idx in range(FT.shape[0]):
            repeat = 0
            try:
                while True:
                    cs = self.circle_search(FT[idx], calibrated[idx], scan)
                    cand = self.computePositionErrorCandidates(cs)
                    ex, ey, edge, _ = self.calculateRMSE(frames[idx], cand, calibrated[idx])
                    calibrated[idx, 0] = calibrated[idx, 0] + ex
                    calibrated[idx, 1] = calibrated[idx, 1] + ey
                    self.rounds[idx] += 1
                    if edge and repeat < 5:
                        repeat += 1
                    else:
                        break
            except Exception:  # noqa: BLE001 - the reference records the frame as failed
                failed.append(idx)
        self.calibrated_positions = calibrated
        self.failed = failed
        if len(failed) != FT.shape[0]:
            src = np.delete(positions, failed, axis=0)
            dst = np.delete(calibrated, failed, axis=0)
            matrix = self.fitCoordinates(src, dst, self.fit_mode)
            return matrix, matrix_transform(positions, matrix.params)
        return SimilarityTransform(np.eye(3)), positions

    @staticmethod
    def fitCoordinates(src, dst, mode):
        """CalibrationFPM.py:745-789."""
        cls = {"Translation": EuclideanTransform}.get(mode, TRANSFORMS.get(mode, EuclideanTransform))
        thresh = np.median(np.abs(dst - src))
        matrix, _ = ransac((src, dst), cls, min_samples=2, residual_threshold=thresh, max_trials=10000)
        if matrix is None:
            raise RuntimeError("no inliers: the calibrated positions do not fit a transform")
        if mode == "Translation":
            matrix = cls(translation=matrix.translation)
        return matrix

    def run(self, ptychogram, positions_pixels):
        """CalibrationFPM.py:830-919 up to the encoder update; returns
        (matrix, NA, entrance pupil diameter, fitted integer positions)."""
        frames = ptychogram.copy()
        initial = positions_pixels - self.No // 2 + self.Np // 2
        FT = self.convertToFourierSpace(frames)
        if not hasattr(self.brightfieldIndices, "__len__"):
            self.brightfieldIndices = self.findBrightfielIndices(frames)
        bf = self.brightfieldIndices
        if self.calibrateRadius:
            _, new = self.findCalibratedRadius(FT[bf], initial[bf])
            self.NA = np.round(new / self.dxp * self.wavelength / self.img_size, 3)
            self.apertRadiusPixel = new
        else:
            self.NA = self.apertRadiusPixel / self.dxp * self.wavelength / self.img_size
        matrix, _ = self.findPositionCalibrationMatrix(frames[bf], FT[bf, :, :], initial[bf, :])
        fitted = matrix_transform(initial, matrix.params)
        epd = self.apertRadiusPixel * self.dxp * 2
        return matrix, self.NA, epd, fitted.astype(int)


def encoder_update(encoder, matrix_params, wavelength, dxo, Np, zled):
    """CalibrationFPM.py:791-828: the calibration matrix in encoder units."""
    conv = -(1 / wavelength) * dxo * Np
    P = np.asarray(matrix_params).copy()
    E = P.copy()
    E[0:2, 2] = np.sign(conv) * P[0:2, 2] * zled / (np.sqrt(conv**2 - P[0, 2] ** 2 - P[1, 2] ** 2))
    return matrix_transform(encoder, E)


def window_and_spectra(frames):
    """The first step alone: windowed frames (float32) and |ifft2c| of them."""
    w = hann_window(frames.shape[1:])
    win = (frames * w[None]).astype(np.float32) if frames.dtype == np.float32 else frames * w[None]
    return win, np.abs(ifft2c(win))


def gaussian_weights(sigma, truncate=4.0):
    """The 1-D weights scipy.ndimage.gaussian_filter uses (radius, weights)."""
    radius = int(truncate * float(sigma) + 0.5)
    x = np.arange(-radius, radius + 1)
    phi = np.exp(-0.5 / (sigma * sigma) * x**2)
    return radius, phi / phi.sum()


def rms_of_candidates(image, F, shifts, position, radius):
    """sqrt(mean((image - |ifft2c(pupil * F)|)^2)) for each (ex, ey) shift."""
    n = image.shape[-1]
    xx, yy = np.mgrid[0:n, 0:n]
    out = []
    for ex, ey in shifts:
        pupil = (((xx - n / 2.0 + (position[0] + ex)) ** 2 + (yy - n / 2.0 + (position[1] + ey)) ** 2)
                 <= radius**2).astype(np.float64)
        est = np.abs(ifft2c(pupil * F))
        out.append(math.sqrt(float(np.mean((image - est) ** 2))))
    return np.asarray(out)
