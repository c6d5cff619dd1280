"""``Simpli``: the user-facing forward-model API of fastpli on the GPU.

Mirrors the parts of ``fastpli.simulation.Simpli`` that drive the forward
model (src/fastpli/simulation/simpli.py:18-187 and the property setters of
src/fastpli/simulation/__simpli.py:97-430): volume and optics properties,
``generate_tissue()``, ``run_simulation()``, the optic and analysis stages,
the tissue / simulation pipelines that write their results to an h5py file
(simpli.py:189-510, duck-typed: any object with h5py's dataset interface)
and ``memory_usage()``.  The compiled back ends are this package's ``_Generator``
and ``_Simulator``.  Device-resident helpers (``*_device``) keep the tissue
in HBM across tilts, which the host API cannot (each reference call re-passes
the tissue from host memory).
"""

import warnings

import numpy as np

from . import objects
from .simulation import _Generator, _Simulator


class Simpli:
    """GPU forward model of 3D-PLI with fastpli's Simpli interface."""

    _FROZEN_OK = True

    def __init__(self, mpi_comm=None):
        if mpi_comm is not None:
            raise NotImplementedError("MPI is not supported: one GPU per process")
        self._dim = None
        self._dim_origin = np.array([0, 0, 0], dtype=float)
        self._voxel_size = None
        self._fiber_bundles = None
        self._filter_rotations = None
        self._flip_z_beam = False
        self._interpolate = "Slerp"
        self._light_intensity = None
        self._pixel_size = None
        self._optical_sigma = None
        self._step_size = 1.0
        self._tilts = None
        self._tissue_refrection = 1.0
        self._background_absorption = 0.0
        self._untilt_sensor_view = True
        self._wavelength = None
        self._noise_model = None
        self._omp_num_threads = 1
        self._verbose = False
        self._gen = _Generator()
        self._sim = _Simulator()
        self._frozen = True

    def __setattr__(self, key, value):
        if getattr(self, "_frozen", False) and not hasattr(self, key):
            raise TypeError(f"{self.__class__.__name__} is a frozen class")
        object.__setattr__(self, key, value)

    # ------------------------------------------------------------ volume ---
    @property
    def dim(self):
        return self._dim

    @dim.setter
    def dim(self, dim):
        dim = np.array(dim)
        if dim.dtype.kind not in "iu":
            raise TypeError("dim is not np.ndarray(int)")
        if dim.size != 3:
            raise TypeError("dim.size != 3")
        if dim.ndim != 1:
            raise TypeError("dim.ndim != 1")
        self._dim = dim.astype(int)

    @property
    def dim_origin(self):
        return self._dim_origin

    @dim_origin.setter
    def dim_origin(self, v):
        self._dim_origin = np.array(v, dtype=float)

    @property
    def voxel_size(self):
        return self._voxel_size

    @voxel_size.setter
    def voxel_size(self, voxel_size):
        # __simpli.py:128-143: keeps the VOI when the voxel size changes
        if voxel_size <= 0:
            raise ValueError("voxel_size <= 0")
        keep = self._voxel_size is not None and self._dim is not None
        if keep:
            v_min, v_max = self.get_voi()
        self._voxel_size = float(voxel_size)
        if keep:
            self.set_voi(v_min, v_max)

    def get_voi(self):
        if self._voxel_size is None:
            raise ValueError("voxel_size is not set, voi can't be calculated")
        if self._dim is None:
            raise ValueError("dim is not set, voi can't be calculated")
        v_min = np.array(self._dim_origin, dtype=float)
        v_max = v_min + self._dim * self._voxel_size
        return v_min, v_max

    def set_voi(self, v_min, v_max):
        v_min = np.array(v_min, dtype=float)
        v_max = np.array(v_max, dtype=float)
        if v_min.ndim != 1 or v_max.ndim != 1:
            raise TypeError("v_min,v_max : ndim != 1")
        if v_min.size != 3 or v_max.size != 3:
            raise TypeError("v_min,v_max : size != 1")
        if np.any(v_min >= v_max):
            raise ValueError("v_min >= v_max")
        if self._voxel_size is None:
            raise TypeError("voxel_size is not set yet")
        self._dim = np.array(np.round((v_max - v_min) / self._voxel_size), dtype=int)
        self._dim_origin = v_min

    # ------------------------------------------------------------ optics ---
    def _scalar(name, conv=float, check=None):
        def get(self):
            return getattr(self, "_" + name)

        def set_(self, v):
            v = conv(v)
            if check:
                check(v)
            object.__setattr__(self, "_" + name, v)
        return property(get, set_)

    def _positive(name):
        def check(v):
            if v <= 0:
                raise ValueError(f"{name} <= 0")
        return check

    light_intensity = _scalar("light_intensity")
    wavelength = _scalar("wavelength")
    background_absorption = _scalar("background_absorption")
    tissue_refrection = _scalar("tissue_refrection")
    step_size = _scalar("step_size")
    verbose = _scalar("verbose", bool)
    untilt_sensor_view = _scalar("untilt_sensor_view", bool)
    flip_z_beam = _scalar("flip_z_beam", bool)
    pixel_size = _scalar("pixel_size", float, _positive("pixel_size"))
    omp_num_threads = _scalar("omp_num_threads", int)

    del _scalar, _positive

    @property
    def filter_rotations(self):
        return self._filter_rotations

    @filter_rotations.setter
    def filter_rotations(self, v):
        v = np.array(v, dtype=float)
        if v.size == 0 or v.ndim != 1:
            raise TypeError("filter_rotations : nx1")
        self._filter_rotations = v

    @property
    def interpolate(self):
        return self._interpolate

    @interpolate.setter
    def interpolate(self, v):
        if v not in ("NN", "Lerp", "Slerp"):
            raise ValueError("Only 'NN', 'Lerp' or 'Slerp' are supported")
        self._interpolate = v

    @property
    def tilts(self):
        return self._tilts

    @tilts.setter
    def tilts(self, tilts):
        if not isinstance(tilts, (list, tuple, np.ndarray)):
            raise TypeError("tilts is not a list or array")
        tilts = np.array(tilts, ndmin=2)
        if tilts.ndim != 2 or tilts.shape[-1] != 2:
            raise TypeError("tilts.shape != nx2")
        self._tilts = tilts

    @property
    def optical_sigma(self):
        return self._optical_sigma

    @optical_sigma.setter
    def optical_sigma(self, v):
        if not isinstance(v, (int, float)):
            raise TypeError("optical_sigma is not a number")
        if v < 0:
            raise ValueError("optical_sigma is < 0")
        self._optical_sigma = v

    @property
    def noise_model(self):
        return self._noise_model

    @noise_model.setter
    def noise_model(self, f):
        if not callable(f):
            raise TypeError("noise model is not callable")
        self._noise_model = f

    @property
    def fiber_bundles(self):
        return self._fiber_bundles

    @fiber_bundles.setter
    def fiber_bundles(self, fbs):
        self._fiber_bundles = None if fbs is None else objects.FiberBundles(fbs)

    def get_dict(self):
        out = {}
        for k, v in self.__dict__.items():
            if k in ("_fiber_bundles", "_gen", "_sim", "_frozen"):
                continue
            if k.startswith("_") and not k.startswith("__"):
                out[k[1:]] = v.tolist() if isinstance(v, np.ndarray) else v
        return out

    def set_dict(self, data):
        for k, v in data.items():
            if k.startswith("_"):
                raise ValueError("member variable cant be set directly")
            if v is not None:
                setattr(self, k, v)
            else:
                warnings.warn("None value in dict detected")

    def memory_usage(self, item="all", unit="MB"):
        """Bytes needed for label + vector (+ distance) per voxel
        (simpli.py:537-571)."""
        if self._dim is None:
            raise ValueError("dim not set")
        n = float(np.prod(self._dim))
        per = {"label": 4, "vector": 12, "all": 16 + 8}[item]
        scale = {"B": 1, "kB": 1e-3, "MB": 1e-6, "GB": 1e-9}[unit]
        return n * per * scale

    # ------------------------------------------------------------ checks ---
    def _check_volume_input(self):
        if self._dim is None:
            raise ValueError("dim not set")
        if self._dim_origin is None:
            raise ValueError("dim_origin not set")
        if self._voxel_size is None:
            raise ValueError("voxel_size not set")

    def _check_generation_input(self):
        if not self._fiber_bundles:
            raise ValueError("fiber_bundles is not set")
        for lys in self._fiber_bundles.layers:
            if lys is None:
                raise ValueError('fiber_bundle properties are "None"')

    def _check_simulation_input(self):
        if self._step_size <= 0:
            raise ValueError("step_size <= 0")
        if self._light_intensity is None:
            raise ValueError("light_intensity not set")
        if self._voxel_size is None:
            raise ValueError("voxel_size not set")
        if self._wavelength is None:
            raise ValueError("wavelength not set")
        if self._filter_rotations is None:
            raise ValueError("filter_rotations not set")

    def _init_pli_setup(self):
        self._check_simulation_input()
        self._sim.set_pli_setup(self._step_size, self._light_intensity,
                                self._voxel_size, self._wavelength,
                                self._tissue_refrection, self._interpolate,
                                self._untilt_sensor_view, self._flip_z_beam,
                                self._filter_rotations)

    def _prepare_generator(self):
        self._check_volume_input()
        self._check_generation_input()
        self._gen.set_volume(self._dim, self._dim_origin, self._voxel_size)
        self._gen.set_fiber_bundles(self._fiber_bundles.as_array(),
                                    [list(l) for l in self._fiber_bundles.layers])

    # -------------------------------------------------------- forward model ---
    def generate_tissue(self, only_tissue=False):
        """simpli.py:61-104 -> (tissue, optical_axis, tissue_properties)."""
        self._prepare_generator()
        tissue, optical_axis, props = self._gen.run_generation(only_tissue)
        props[0, 1] = self._background_absorption
        if not np.any(tissue):
            warnings.warn("All labels are 0. Usually this means, that the VOI "
                          "contains no fiber_bundles or that the voxel_size is to "
                          "large.", UserWarning)
        return tissue, optical_axis, props

    def run_simulation(self, tissue, optical_axis, tissue_properties, theta, phi):
        """simpli.py:125-187 -> images float64 [X, Y, n_rho]."""
        self._check_volume_input()
        self._init_pli_setup()
        tissue_properties = np.array(tissue_properties)
        if tissue_properties.ndim != 2:
            raise ValueError("tissue_properties.ndim !=2")
        if tissue_properties.shape[1] != 2:
            raise ValueError("tissue_properties.shape[1] != 2")
        tissue = np.asarray(tissue)
        optical_axis = np.asarray(optical_axis)
        if tissue.ndim != 3:
            raise ValueError("tissue.ndim != 3")
        if optical_axis.ndim != 4:
            raise ValueError("optical_axis.ndim != 4")
        if optical_axis.shape[3] != 3:
            raise ValueError("optical_axis.shape[3] != 3")
        if tuple(tissue.shape) != tuple(optical_axis.shape[:-1]):
            raise ValueError("not np.equal(tissue.shape, optical_axis.shape[:-1])")
        if tissue.dtype != np.int32:
            warnings.warn("tissue is copied", UserWarning)
        if optical_axis.dtype != np.float32:
            warnings.warn("optical_axis is copied", UserWarning)
        images = self._sim.run_simulation(self._dim, tissue, optical_axis,
                                          tissue_properties, theta, phi)
        if np.min(images.flatten()) < 0:
            raise ValueError("intensity < 0 detected")
        return images

    def apply_epa(self, data, mask=None):
        """__simpli.py:597-621: transmittance, direction, retardation (NaN
        outside ``mask``)."""
        from . import analysis
        t, d, r = analysis.epa(data)
        if mask is not None:
            inv = ~np.asarray(mask, bool) if not hasattr(mask, "is_cuda") else ~mask
            t[inv], d[inv], r[inv] = float("nan"), float("nan"), float("nan")
        return t, d, r

    def apply_rofl(self, data, mask=None, mp_pool=None, grad_mode=False):
        """ROFL of every pixel (__simpli.py:623-705): data [5, X, Y, n_rho]
        for the tilts (0,0), (tau,0), (tau,90), (tau,180), (tau,270) degrees.
        Returns directionmap, inclmap, trelmap, (dirdevmap, incldevmap,
        treldevmap, funcmap, itermap); pixels outside ``mask`` are NaN (the
        reference leaves them uninitialised).  numpy data -> numpy maps, CUDA
        tensor -> CUDA maps.  ``mp_pool`` is accepted and unused."""
        from . import analysis
        if self._tilts is None:
            raise ValueError("tilts not set")
        tl = self._tilts
        if tl.shape[0] != 5 or np.any(tl[:, 1] != np.deg2rad([0, 0, 90, 180, 270])) or \
                tl[0, 0] != 0 or np.any(tl[1:, 0] != tl[1, 0]):
            raise ValueError("tilts not suitable for ROFL")
        tilt_angle = tl[1, 0]
        on_device = hasattr(data, "is_cuda") and data.is_cuda
        if on_device:
            torch = analysis._torch()
            out_dtype = torch.float32 if data.element_size() <= 4 else torch.float64
            d = data
        else:
            data = np.asarray(data)
            out_dtype = np.float32 if data.itemsize <= 4 else np.float64
            import torch
            d = torch.from_numpy(np.ascontiguousarray(data, np.float64)).cuda() \
                if data.ndim == 4 else data
        if d.ndim != 4:
            raise TypeError("data: np.array([tilts,x,y,stack])")
        if d.shape[0] != 5:
            raise ValueError("data need 1 + 4 measurements")
        if d.shape[-1] <= 3:
            raise ValueError("data needs at least 3 equidistant rotations")
        out = analysis.rofl_device(d, tilt_angle, 3, 0, grad_mode, mask)
        maps = [out[:, :, i] for i in range(8)]
        if on_device:
            maps = [m.to(out_dtype) for m in maps]
        else:
            maps = [m.cpu().numpy().astype(out_dtype) for m in maps]
        return maps[0], maps[1], maps[2], tuple(maps[3:])

    # ---------------------------------------------------------------- optic ---
    def apply_optic_resample(self, data, shift=(0, 0), mp_pool=None):
        """Gaussian blur + block-average resample of every polarizer angle
        (__simpli.py:495-550).  ``data`` numpy [X, Y(, n_rho)] (host API) or a
        float64 CUDA tensor (stays on the device).  ``mp_pool`` is accepted
        and unused: all angles go to the GPU in one call."""
        from . import optic
        if self._optical_sigma is None:
            raise ValueError("optical_sigma is None")
        if self._voxel_size is None:
            raise ValueError("voxel_size not set")
        if self._pixel_size is None:
            raise ValueError("pixel_size not set")
        on_device = hasattr(data, "is_cuda") and data.is_cuda
        if not on_device:
            data = np.atleast_3d(np.array(data))
        elif data.dim() == 2:
            data = data[:, :, None]
        if data.ndim > 3:
            raise TypeError("data can be 1d, 2d or 3d")
        shift = np.array(shift, int)
        if shift.size != 2 or shift.ndim != 1:
            raise TypeError("shift has to be (x,y)")
        if shift[0] > 0 and shift[1] > 0:
            data = data[shift[0]:, shift[1]:, ...]
        scale = self._voxel_size / self._pixel_size
        size = np.array(np.round(np.array(data.shape[0:2]) * scale), dtype=int)
        if np.amin(size) == 0:
            raise ValueError(f"voxel_size {self._voxel_size}, pixel_size {self._pixel_size} "
                             f"and data shape {tuple(data.shape[0:2])} result in optical "
                             f"image size of {size}")
        if on_device:
            out = optic.filter_resample_device(data.contiguous().double(),
                                               self._optical_sigma, scale)
            return out.squeeze()
        return np.squeeze(optic.filter_resample(data, self._optical_sigma, scale))

    def apply_optic(self, data, mp_pool=None):
        """Resample, then the noise model (__simpli.py:462-489): returns
        (resampled, noisy).  With a NegativeBinomialNoise model and device
        data the noise is drawn on the device as well."""
        from . import optic
        if self._noise_model is None:
            raise ValueError("noise_model not set")
        resampled = self.apply_optic_resample(data, mp_pool=mp_pool)
        on_device = hasattr(resampled, "is_cuda") and resampled.is_cuda
        lo = float(resampled.min()) if on_device else np.amin(resampled)
        if lo < 0:
            raise AssertionError("intensity < 0 detected")
        if on_device:
            if isinstance(self._noise_model, optic.NegativeBinomialNoise):
                return resampled, self._noise_model.device(resampled)
            import torch
            noisy = optic.add_noise(resampled.cpu().numpy(), self._noise_model)
            return resampled, torch.from_numpy(np.asarray(noisy, np.float64)).to(resampled.device)
        return resampled, optic.add_noise(resampled, self._noise_model)

    # ------------------------------------------------- pipelines and I/O ---
    def _print(self, msg):
        if self._verbose:
            print(msg)

    def save_parameter_h5(self, h5f, script=None):
        """Parameters as attributes of an h5py file or group
        (__simpli.py:450-460)."""
        import sys
        from . import __version__
        h5f.attrs["fastpli/simpli"] = str(self.get_dict())
        h5f.attrs["fastpli/version"] = __version__
        h5f.attrs["fastpli/compiler"] = "nvcc sm_103a (fastpli_gb300)"
        h5f.attrs["fastpli/libraries"] = "fastpli_gb300"
        h5f.attrs["fastpli/pip_freeze"] = ""
        h5f.attrs["fastpli/system"] = sys.version
        if script:
            h5f.attrs["script"] = script.encode().decode("ascii", "ignore")

    def crop_tilt_pixel(self):
        """Image pixels at each border the tilts can reach outside the
        volume (simpli.py:245-261)."""
        if not self._untilt_sensor_view:
            raise ValueError("currently only for untilt_sensor_view=True")
        if self._voxel_size is None:
            raise ValueError("voxel_size is not set")
        if self._pixel_size is None:
            raise ValueError("pixel_size is not set")
        if self._tilts is None:
            raise ValueError("tilts are not set")
        return int(np.ceil(np.tan(np.max(np.abs(self._tilts[:, 0]))) * self._dim[-1] / 2 *
                           self._voxel_size / self._pixel_size))

    def crop_tilt_voxel(self):
        """crop_tilt_pixel in voxels (simpli.py:263-268)."""
        return int(np.round(self.crop_tilt_pixel() * self._pixel_size / self._voxel_size))

    def add_crop_tilt_halo(self):
        """Widen the volume by the tilt halo (simpli.py:270-274)."""
        d = self.crop_tilt_voxel()
        self.dim_origin[:2] -= d * self.voxel_size
        self.dim[:2] += 2 * d

    def rm_crop_tilt_halo(self, data):
        """Remove the halo from images (simpli.py:276-282)."""
        d = self.crop_tilt_voxel()
        if d == 0:
            return data
        return data[d:-d, d:-d, :]

    def run_tissue_pipeline(self, h5f=None, script=None, save=("tissue", "optical_axis")):
        """generate_tissue() with its results written to ``h5f`` (an h5py
        file or anything with its create_dataset / item interface)
        (simpli.py:189-243)."""
        self._print("Run tissue pipeline")
        self._check_volume_input()
        self._check_generation_input()
        save = list(save)
        if script:
            self.save_parameter_h5(h5f, script)
        if "all" in save or "simulation" in save:
            save = save + ["tissue", "optical_axis"]
        tissue, optical_axis, tissue_properties = self.generate_tissue()
        if h5f and "tissue" in save:
            dset = h5f.create_dataset("tissue/tissue", tissue.shape, dtype=np.uint16,
                                      compression="gzip", compression_opts=1)
            dset[:] = tissue
        if h5f and "optical_axis" in save:
            dset = h5f.create_dataset("tissue/optical_axis", optical_axis.shape,
                                      dtype=np.float32, compression="gzip",
                                      compression_opts=1)
            dset[:] = optical_axis
        if h5f and "tissue" in save:
            h5f["tissue/properties"] = tissue_properties
        return tissue, optical_axis, tissue_properties

    def _rofl_tilts_ok(self):
        tl = self._tilts
        return not (np.any(tl[:, 1] != np.deg2rad([0, 0, 90, 180, 270])) or tl[0, 0] != 0 or
                    np.any(tl[1:, 0] != tl[1, 0]))

    def run_simulation_pipeline(self, tissue, optical_axis, tissue_properties, h5f=None,
                                save=("data", "optic", "epa", "mask", "rofl"),
                                crop_tilt=False, mp_pool=None):
        """Every tilt: march, optic, epa; then the pseudo mask and ROFL, with
        results written to ``h5f`` (simpli.py:284-438).  Returns
        (tilting_stack, (rofl_direction, rofl_incl, rofl_t_rel), fom)."""
        from . import analysis
        self._print("Run simulation pipeline")
        save = list(save)
        if "all" in save or "simulation" in save:
            save = save + ["data", "resample", "optic", "epa", "mask", "rofl"]
        if self._tilts is None:
            raise ValueError("tilts is not set")
        if self._optical_sigma is None:
            raise ValueError("optical_sigma is not set")
        flag_rofl = self._rofl_tilts_ok()
        if not flag_rofl:
            warnings.warn("Tilts not suitable for ROFL. Skipping analysis")

        def put(name, value, theta=None, phi=None):
            h5f[name] = value
            if theta is not None:
                h5f[name].attrs["theta"] = theta
                h5f[name].attrs["phi"] = phi

        stack = [None] * len(self._tilts)
        for t, (theta, phi) in enumerate(self._tilts):
            self._print(f"Tilt {t}: theta: {np.rad2deg(theta):.1f} deg, phi: "
                        f"{np.rad2deg(phi):.1f} deg")
            images = self.run_simulation(tissue, optical_axis, tissue_properties, theta, phi)
            if crop_tilt:
                images = self.rm_crop_tilt_halo(images)
            if h5f and "data" in save:
                put(f"simulation/data/{t}", images, theta, phi)
            img_res, img_noise = self.apply_optic(images, mp_pool=mp_pool)
            if h5f and "resample" in save:
                put(f"simulation/resample/{t}", img_res, theta, phi)
            if h5f and "optic" in save:
                put(f"simulation/optic/{t}", img_noise, theta, phi)
            if h5f and "epa" in save:
                epa = self.apply_epa(img_noise)
                for name, v in zip(("transmittance", "direction", "retardation"), epa):
                    put(f"analysis/epa/{t}/{name}", v, theta, phi)
            stack[t] = img_noise
        if h5f and "mask" in save:
            mask = np.sum(tissue, 2) > 0
            mask = self.apply_optic_resample(1.0 * mask, mp_pool=mp_pool) > 0.1
            h5f["simulation/optic/mask"] = np.uint8(mask)
        stack = np.array(stack)
        while stack.ndim < 4:
            stack = np.expand_dims(stack, axis=-2)
        rofl = (None,) * 3
        conf = (None,) * 5
        if flag_rofl:
            d, i, tr, conf = self.apply_rofl(stack, mask=None, mp_pool=mp_pool)
            rofl = (d, i, tr)
        if h5f and flag_rofl and "rofl" in save:
            h5f["analysis/rofl/direction"] = rofl[0]
            h5f["analysis/rofl/inclination"] = rofl[1]
            h5f["analysis/rofl/t_rel"] = rofl[2]
        if h5f and flag_rofl and "rofl_conf" in save:
            for name, v in zip(("direction_conf", "inclination_conf", "t_rel_conf", "func",
                                "n_iter"), conf):
                h5f[f"analysis/rofl/{name}"] = v
        fom = analysis.fom_hsv_black(rofl[0], rofl[1]) if flag_rofl else None
        return stack, rofl, fom

    def run_pipeline(self, h5f=None, script=None,
                     save=("tissue", "optical_axis", "data", "optic", "epa", "mask", "rofl"),
                     crop_tilt=False, mp_pool=None):
        """Tissue then simulation pipeline (simpli.py:440-510).  Returns
        ((tissue, optical_axis, tissue_properties), tilting_stack,
        (rofl_direction, rofl_incl, rofl_t_rel), fom)."""
        self._print("Run pipeline")
        save = list(save)
        if "all" in save:
            save = ["tissue", "optical_axis", "data", "optic", "epa", "mask", "rofl"]
        if "tissue" in save:
            save = save + ["tissue", "optical_axis"]
        if "simulation" in save:
            save = save + ["data", "optic", "epa", "mask", "rofl"]
        self._check_volume_input()
        self._check_generation_input()
        self._check_simulation_input()
        if self._tilts is None:
            raise ValueError("tilts is not set")
        if self._optical_sigma is None:
            raise ValueError("optical_sigma is not set")
        if h5f:
            self.save_parameter_h5(h5f, script)
        tissue, optical_axis, props = self.run_tissue_pipeline(h5f=h5f, script=script,
                                                               save=save)
        stack, rofl, fom = self.run_simulation_pipeline(tissue, optical_axis, props, h5f=h5f,
                                                        save=save, crop_tilt=crop_tilt,
                                                        mp_pool=mp_pool)
        return (tissue, optical_axis, props), stack, rofl, fom

    def apply_epa_device(self, data, mask=None):
        """epa of a device image stack in FP64 (epa.py:9-45) -> (t, d, r)."""
        from . import optic
        t, d, r = optic.epa_device(data)
        if mask is not None:
            t[~mask], d[~mask], r[~mask] = 0, 0, 0
        return t, d, r

    # ------------------------------------------------- device-resident path ---
    def generate_tissue_device(self, only_tissue=False, stream=None):
        """Voxelize into HBM: (label, vector) torch CUDA tensors + props."""
        self._prepare_generator()
        label, vector, props, _ = self._gen.run_generation_device(only_tissue, stream)
        props = props.copy()
        props[0, 1] = self._background_absorption
        return label, vector, props

    def run_simulation_device(self, label, vector, tissue_properties, theta, phi,
                              epa=False, stream=None):
        """March device-resident tissue (no host copies)."""
        self._check_volume_input()
        self._init_pli_setup()
        return self._sim.run_simulation_device(self._dim, label, vector,
                                               tissue_properties, theta, phi,
                                               epa=epa, stream=stream)

    def run_tilts_device(self, label, vector, tissue_properties, tilts=None,
                         epa=False, stream=None):
        """All tilts of ``self.tilts`` on resident tissue -> list of results
        (the tilts' marches overlap on the GPU; each result is the one
        run_simulation_device gives)."""
        tilts = self._tilts if tilts is None else np.array(tilts, ndmin=2)
        if tilts is None:
            raise ValueError("tilts not set")
        self._check_volume_input()
        self._init_pli_setup()
        return self._sim.run_tilts_device(self._dim, label, vector, tissue_properties,
                                          tilts, epa=epa, stream=stream)
