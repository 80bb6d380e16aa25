"""Model-development front end: parameters, datasets, GPU fit, errors, files.

`Pypolymlp` mirrors the reference's class of the same name
(src/pypolymlp/mlp_dev/pypolymlp.py:34-850) for the structure-list entry point:
`set_params` takes the settings of `set_all_params` (core/params_utils.py:141-245:
elements, cutoff, model type, polynomial order, Gaussian radial functions as two
linspaces or `n_gaussians`, `distance`-conditioned radial functions, ridge
alphas 10^linspace(reg_alpha_params), invariant order and l_max, atomic
energies in eV or Hartree, spins); `set_datasets_structures` takes training and
test structures (`calculator.PolymlpStructure`, atom types set from element
names) with energies in eV per cell, forces (3, n_atom) and stress tensors
(3, 3) in eV per cell, turning force and stress fitting off where the data are
absent (pypolymlp.py:264-271) and subtracting the atomic energies
(dataset_utils.py:300-305); `fit`, `fit_cg`, `run`, `estimate_error` and
`fit_learning_curve` call the GPU regression (`regression.fit`, `fit_cg`,
`fit_learning_curve`) and `accuracy.PolymlpEvalAccuracy`; `save_mlp`,
`load_mlp`, `save_params` and `save_errors` write the reference's files.

`precision` selects the rows and the Gram: PG_FP64 (default; the reference's
arithmetic) or PG_MIXED (FP32 rows, and their Gram on the tensor cores from
fixed-point BF16 slices, accurate to ~1e-12, solved directly in FP64).
`set_datasets_vasp` and `set_multiple_datasets_vasp` read vasprun.xml files
(`io_vasp`); the reference's electron, SSCHA, phono3py and property-yaml
dataset readers are not part of this module.
"""

from __future__ import annotations

from typing import Optional, Sequence

import numpy as np

from pypolymlp_gb300 import _ffi
from pypolymlp_gb300.calculator import PolymlpStructure, replace_types
from pypolymlp_gb300.params import make_params_dict

def _strtobool(v) -> bool:
    t = str(v).strip().lower()
    if t in ("y", "yes", "t", "true", "on", "1"):
        return True
    if t in ("n", "no", "f", "false", "off", "0"):
        return False
    raise ValueError(f"invalid truth value {v!r}")


HARTREE_TO_EV = 27.211386245981  # the reference's conversion (core/units.py:31)


class Pypolymlp:
    def __init__(self, verbose: bool = False, precision: int = _ffi.PG_FP64):
        self._verbose = verbose
        self._precision = precision
        self._params: Optional[dict] = None
        self._alphas = None
        self._atomic_energy = None
        self._train = self._test = None
        self._result = None
        self._coeffs = self._scales = None
        self._error_train = self._error_test = None
        self._learning_log = None
        self._hybrid: list = []
        self._cumulative = None

    # -- parameters -----------------------------------------------------------------
    def set_params(self, params: Optional[dict] = None, elements: Optional[Sequence[str]] = None,
                   include_force: bool = True, include_stress: bool = True, cutoff: float = 6.0,
                   model_type: int = 4, max_p: int = 2, feature_type: str = "gtinv",
                   gaussian_params1=(1.0, 1.0, 1), gaussian_params2=(0.0, 5.0, 7),
                   n_gaussians: Optional[int] = None, distance: Optional[dict] = None,
                   reg_alpha_params=(-3.0, 1.0, 5), gtinv_order: int = 3, gtinv_maxl=(4, 4, 2, 1, 1),
                   gtinv_version: int = 1, atomic_energy_unit: str = "eV",
                   atomic_energy: Optional[Sequence[float]] = None, enable_spins: Optional[Sequence[bool]] = None):
        alphas = [10.0 ** a for a in np.linspace(reg_alpha_params[0], reg_alpha_params[1],
                                                 round(reg_alpha_params[2]))]
        # a new first model drops the models appended to the previous one
        self._hybrid, self._cumulative = [], None
        if params is not None:
            self._params = params
            self._alphas = params.get("alphas") or alphas
            n = len(params.get("spin_elements", {}).get("elements", params["elements"]))
            self._atomic_energy = self._expand_atomic_energy(params, [0.0] * n)
            return self
        if elements is None:
            raise RuntimeError("elements are required")
        n_type = len(elements)
        if atomic_energy is None:
            atomic_energy = [0.0] * n_type
        elif len(atomic_energy) != n_type:
            raise ValueError("one atomic energy per element")
        if atomic_energy_unit == "Hartree":
            atomic_energy = [e * HARTREE_TO_EV for e in atomic_energy]
        self._params = make_params_dict(
            n_type=n_type, cutoff=cutoff, model_type=model_type, max_p=max_p, feature_type=feature_type,
            gaussian_params1=gaussian_params1, gaussian_params2=gaussian_params2, gtinv_order=gtinv_order,
            gtinv_maxl=gtinv_maxl, gtinv_version=gtinv_version, elements=list(elements),
            include_force=include_force, include_stress=include_stress, alphas=alphas, enable_spins=enable_spins,
            n_gaussians=n_gaussians, distance=distance)
        self._alphas = alphas
        self._atomic_energy = self._expand_atomic_energy(self._params, list(atomic_energy))
        return self

    def append_hybrid_params(self, **kwargs):
        """Add one more model over the same elements (a hybrid; mlp_dev/pypolymlp.py:152-237):
        the settings of `set_params`; the datasets and alphas stay those of the first model."""
        if self._params is None:
            raise RuntimeError("Set the first model's parameters before appending hybrid ones.")
        first = (self._params, self._alphas, self._atomic_energy, self._hybrid)
        self.set_params(**kwargs)
        extra = self._params
        self._params, self._alphas, self._atomic_energy, self._hybrid = first
        if list(extra["elements"]) != list(self._params["elements"]):
            raise ValueError("hybrid models here share the first model's elements")
        self._hybrid = list(self._hybrid) + [extra]
        return self

    @property
    def _models(self) -> list:
        return [self._params] + list(self._hybrid)

    def _single_model_only(self, what: str):
        if self._hybrid:
            raise RuntimeError(f"{what} fits one model; this Pypolymlp holds a hybrid of {len(self._models)} "
                               "models (use fit or run without use_cg)")

    @staticmethod
    def _expand_atomic_energy(params: dict, per_element: list) -> np.ndarray:
        """Atomic energy per atom type (spin-split elements repeat theirs)."""
        sp = params.get("spin_elements")
        if not sp:
            return np.asarray(per_element, dtype=np.float64)
        out = np.zeros(int(params["n_type"]))
        for e, types in zip(per_element, sp["types"]):
            out[types] = e
        return out

    # -- datasets -------------------------------------------------------------------
    def set_datasets_structures(self, train_structures: Sequence[PolymlpStructure],
                                test_structures: Sequence[PolymlpStructure], train_energies, test_energies,
                                train_forces: Optional[Sequence] = None, test_forces: Optional[Sequence] = None,
                                train_stresses=None, test_stresses=None):
        if self._params is None:
            raise RuntimeError("Set parameters before datasets.")
        for forces, stresses in ((train_forces, train_stresses), (test_forces, test_stresses)):
            if forces is None:
                self._params["include_force"] = self._params["include_stress"] = False
            if stresses is None:
                self._params["include_stress"] = False

        self._train = [self._dataset(train_structures, train_energies, train_forces, train_stresses, "data1")]
        self._test = [self._dataset(test_structures, test_energies, test_forces, test_stresses, "data2")]
        return self

    def load_parameter_file(self, file_params: str, train_ratio: float = 0.9, prefix: Optional[str] = None):
        """Settings and vasprun datasets of a polymlp.in file
        (core/parser_polymlp_params.py, parser_infile.py:15-30, dataset.py:119-140):
        model keys as `set_params` takes them, `distance A B d1 d2 ...` lines,
        `atomic_energy`, `reg_alpha_params`, `include_force` / `include_stress`,
        and `train_data` / `test_data` / `data` / `data_md` lines "glob [include_force
        [weight]]" (files sorted; `data` split by file with the reference's rule
        into "Train_<glob>" and "Test_<glob>", `data_md` - one MD vasprun.xml - split
        by step the same way, parser_polymlp_params.py:253-284, dataset.py:142-205;
        other datasets are named by their glob; `prefix` is prepended to the
        path)."""
        import glob

        from pypolymlp_gb300.io_vasp import split_train_test

        kv, distance, data_lines = {}, {}, []
        with open(file_params) as f:
            for line in f:
                d = line.split("#", 1)[0].split()
                if len(d) < 2:
                    continue
                if d[0] == "distance":
                    distance[(d[1], d[2])] = [float(v) for v in d[3:]]
                elif "data" in d[0] and "dataset_type" not in d[0]:
                    data_lines.append(d)
                else:
                    kv[d[0]] = d[1:]
        if kv.get("dataset_type", ["vasp"])[0] != "vasp":
            raise NotImplementedError("only vasp datasets are read from parameter files")

        def one(key, conv, default=None):
            return conv(kv[key][0]) if key in kv else default

        def triple(key, default):
            if key not in kv:
                return default
            a, b, n = kv[key][:3]
            return float(a), float(b), int(float(n))

        kw = dict(elements=kv["elements"], include_force=one("include_force", _strtobool, True),
                  include_stress=one("include_stress", _strtobool, True), cutoff=one("cutoff", float, 6.0),
                  model_type=one("model_type", int, 4), max_p=one("max_p", int, 2),
                  feature_type=one("feature_type", str, "gtinv"),
                  gaussian_params1=triple("gaussian_params1", (1.0, 1.0, 1)),
                  gaussian_params2=triple("gaussian_params2", (0.0, 5.0, 7)),
                  n_gaussians=one("n_gaussians", int), distance=distance or None,
                  reg_alpha_params=triple("reg_alpha_params", (-3.0, 1.0, 5)),
                  gtinv_order=one("gtinv_order", int, 3),
                  gtinv_maxl=tuple(int(v) for v in kv.get("gtinv_maxl", [4, 4, 2, 1, 1])),
                  gtinv_version=one("gtinv_version", int, 1),
                  atomic_energy=[float(v) for v in kv["atomic_energy"]] if "atomic_energy" in kv else None,
                  enable_spins=[_strtobool(v) for v in kv["enable_spins"]] if "enable_spins" in kv else None)
        self.set_params(**kw)
        self._train, self._test = [], []
        for d in data_lines:
            tag, name = d[0], d[1]
            files = sorted(glob.glob(name if prefix is None else prefix + "/" + name))
            force = _strtobool(d[2]) if len(d) > 2 else self._params["include_force"]
            force = force and self._params["include_force"]
            stress = force and self._params["include_stress"]
            weight = float(d[3]) if len(d) > 3 else 1.0
            if tag == "train_data":
                self._train.append(self._vasp_dataset(files, name, force, stress, weight))
            elif tag == "test_data":
                self._test.append(self._vasp_dataset(files, name, force, stress, weight))
            elif tag == "data":
                tr, te = split_train_test(files, train_ratio)
                self._train.append(self._vasp_dataset(tr, "Train_" + name, force, stress, weight))
                self._test.append(self._vasp_dataset(te, "Test_" + name, force, stress, weight))
            elif tag == "data_md":
                from pypolymlp_gb300.io_vasp import parse_properties_from_vaspruns, split_ids_train_test

                sts, (e, f, st6) = parse_properties_from_vaspruns(files, verbose=self._verbose)
                tr, te = split_ids_train_test(len(sts), train_ratio)
                for ids, nm, out in ((tr, "Train_" + name, self._train), (te, "Test_" + name, self._test)):
                    out.append(self._dataset([sts[i] for i in ids], e[ids], [f[i] for i in ids], st6[ids], nm,
                                             force, stress, weight))
        return self

    def _dataset(self, structures, energies, forces, stresses, name, include_force=None, include_stress=None,
                 weight=1.0):
        """regression.Dataset of structures typed by the model's element order,
        atomic energies subtracted, stresses as (xx, yy, zz, xy, yz, zx)."""
        from pypolymlp_gb300.regression import Dataset

        elements = list(self._params["elements"])
        types = [replace_types(st, elements) for st in structures]
        axis = [np.asarray(st.axis, dtype=np.float64) for st in structures]
        pos = [(a @ np.asarray(st.positions, dtype=np.float64)).T for a, st in zip(axis, structures)]
        e = np.asarray(energies, dtype=np.float64) - np.array([self._atomic_energy[t].sum() for t in types])
        f = None if forces is None else [np.asarray(x, dtype=np.float64).T for x in forces]
        s = None
        if stresses is not None:
            t = np.asarray(stresses, dtype=np.float64).reshape(-1, 3, 3)
            s = np.stack([t[:, 0, 0], t[:, 1, 1], t[:, 2, 2], t[:, 0, 1], t[:, 1, 2], t[:, 2, 0]], axis=1)
        force = self._params["include_force"] if include_force is None else include_force
        stress = self._params["include_stress"] if include_stress is None else include_stress
        return Dataset(axis, pos, types, e, f, s, include_force=force, include_stress=stress, weight=weight, name=name)

    def _vasp_dataset(self, files, name, include_force=None, include_stress=None, weight=1.0):
        from pypolymlp_gb300.io_vasp import parse_properties_from_vaspruns

        sts, (e, f, s) = parse_properties_from_vaspruns(sorted(files), verbose=self._verbose)
        return self._dataset(sts, e, f, s, name, include_force, include_stress, weight)

    def set_datasets_vasp(self, train_vaspruns: Optional[Sequence[str]] = None,
                          test_vaspruns: Optional[Sequence[str]] = None, vaspruns=None, train_ratio: float = 0.9):
        """One training and one test dataset from vasprun.xml files (dataset.py:567-637):
        given lists, or one list split by the reference's rule (files sorted
        first), or one MD vasprun whose steps are split."""
        from pypolymlp_gb300.io_vasp import parse_properties_from_vaspruns, split_ids_train_test, split_train_test

        if self._params is None:
            raise RuntimeError("Set parameters before datasets.")
        if train_vaspruns is not None and test_vaspruns is not None:
            self._train = [self._vasp_dataset(train_vaspruns, "data1")]
            self._test = [self._vasp_dataset(test_vaspruns, "data2")]
        elif isinstance(vaspruns, str):
            sts, (e, f, s) = parse_properties_from_vaspruns([vaspruns], verbose=self._verbose)
            tr, te = split_ids_train_test(len(sts), train_ratio)
            self._train = [self._dataset([sts[i] for i in tr], e[tr], [f[i] for i in tr], s[tr], "data1")]
            self._test = [self._dataset([sts[i] for i in te], e[te], [f[i] for i in te], s[te], "data2")]
        else:
            tr_files, te_files = split_train_test(sorted(vaspruns), train_ratio)
            self._train = [self._vasp_dataset(tr_files, "data1")]
            self._test = [self._vasp_dataset(te_files, "data2")]
        return self

    def set_multiple_datasets_vasp(self, train_vaspruns: Sequence[Sequence[str]],
                                   test_vaspruns: Sequence[Sequence[str]]):
        """Several training and test datasets, named data1, data2, ... in each list."""
        if self._params is None:
            raise RuntimeError("Set parameters before datasets.")
        self._train = [self._vasp_dataset(f, f"data{i + 1}") for i, f in enumerate(train_vaspruns)]
        self._test = [self._vasp_dataset(f, f"data{i + 1}") for i, f in enumerate(test_vaspruns)]
        return self

    def _ready(self):
        if self._params is None or self._train is None or self._test is None:
            raise RuntimeError("Set parameters and datasets before using fit.")

    # -- fitting --------------------------------------------------------------------
    def fit(self, batch_size: Optional[int] = None, verbose: Optional[bool] = None):
        """Ridge regression over the alphas on the GPU Gram (batch_size: the
        device batches are sized by memory; the argument is accepted and unused)."""
        from pypolymlp_gb300 import regression

        self._ready()
        if len(self._models) > 1:
            from pypolymlp_gb300.hybrid import fit_hybrid

            res, self._cumulative = fit_hybrid(self._models, self._train, self._test, self._alphas,
                                               precision=self._precision)
            return self._set_result(res)
        res = regression.fit(self._params, self._train, self._test, self._alphas, precision=self._precision)
        return self._set_result(res)

    def fit_standard(self, verbose: Optional[bool] = None):
        return self.fit(verbose=verbose)

    def fit_cg(self, gtol: float = 1e-2, max_iter: Optional[int] = None, verbose: Optional[bool] = None):
        from pypolymlp_gb300 import regression

        self._ready()
        self._single_model_only("fit_cg")
        res = regression.fit_cg(self._params, self._train, self._test, self._alphas, gtol=gtol, max_iter=max_iter,
                                precision=self._precision)
        return self._set_result(res)

    def fit_sgd(self, verbose: Optional[bool] = None):
        raise NotImplementedError("SGD not available.")

    def _set_result(self, res):
        self._result = res
        self._scales = np.asarray(res.scales, dtype=np.float64)
        self._coeffs = np.asarray(res.coeffs, dtype=np.float64)
        return self

    def estimate_error(self, log_energy: bool = False, file_path: str = "./", verbose: Optional[bool] = None):
        from pypolymlp_gb300.accuracy import PolymlpEvalAccuracy

        if self._coeffs is None:
            raise RuntimeError("Regression must be performed before estimating errors.")
        if len(self._models) > 1:
            return self._estimate_error_hybrid()
        acc = PolymlpEvalAccuracy(self._params, self._coeffs / self._scales, verbose=self._verbose)
        self._error_train = acc.compute_error(self._train, log_energy=log_energy, path_output=file_path, tag="train")
        self._error_test = acc.compute_error(self._test, log_energy=log_energy, path_output=file_path, tag="test")
        return self

    def _estimate_error_hybrid(self):
        """Errors of the summed models (hybrid.PropertiesHybrid on the GPU)."""
        from pypolymlp_gb300.accuracy import prediction_errors
        from pypolymlp_gb300.hybrid import PropertiesHybrid

        bounds = [0] + list(self._cumulative)
        c = self._coeffs / self._scales
        ph = PropertiesHybrid(self._models, [c[bounds[k]:bounds[k + 1]] for k in range(len(self._models))],
                              _ffi.PG_FP64)

        def errors(datasets):
            out = {}
            for d in datasets:
                e, f, s = ph.eval_multiple(d.axis, [np.asarray(x).T for x in d.positions], d.types)
                out[d.name], _ = prediction_errors(d, e, f, s)
            return out

        self._error_train, self._error_test = errors(self._train), errors(self._test)
        return self

    def run(self, batch_size: Optional[int] = None, use_cg: bool = False, gtol: float = 1e-2,
            max_iter: Optional[int] = None, verbose: Optional[bool] = None):
        if use_cg:
            self.fit_cg(gtol=gtol, max_iter=max_iter)
        else:
            self.fit(batch_size=batch_size)
        return self.estimate_error()

    def fit_learning_curve(self, verbose: Optional[bool] = None):
        from pypolymlp_gb300 import regression

        self._ready()
        self._single_model_only("fit_learning_curve")
        self._learning_log = regression.fit_learning_curve(self._params, self._train, self._test, self._alphas,
                                                           precision=self._precision)
        return self

    def save_learning_curve(self, filename: str = "polymlp_learning_curve.dat"):
        """One line per (training size, test dataset): n, energy RMSE (meV/atom),
        force RMSE (eV/angstrom), stress RMSE, as utils_learning_curve.py:4-15."""
        with open(filename, "w") as f:
            print("# n_str, RMSE(energy, meV/atom) RMSE(force, eV/ang), RMSE(stress)", file=f)
            for n, err in self._learning_log:
                print(n, err["energy"] * 1000, err["force"], err["stress"], file=f)
        return self

    # -- files ----------------------------------------------------------------------
    def save_mlp(self, filename: str = "polymlp.yaml"):
        from pypolymlp_gb300.io_polymlp import save_mlp_yaml

        if self._coeffs is None:
            raise RuntimeError("No polymlp has been developed.")
        if len(self._models) == 1:
            save_mlp_yaml(self._params, self._coeffs, self._scales, filename)
            return self
        # a hybrid: filename.1, filename.2, ... with each model's columns (pypolymlp.py:710-719)
        bounds = [0] + list(self._cumulative)
        for k, p in enumerate(self._models):
            sl = slice(bounds[k], bounds[k + 1])
            save_mlp_yaml(p, self._coeffs[sl], self._scales[sl], f"{filename}.{k + 1}")
        return self

    def load_mlp(self, filename: str = "polymlp.yaml"):
        from pypolymlp_gb300.io_polymlp import load_mlp

        self._params, coeffs = load_mlp(filename)
        self._hybrid, self._cumulative = [], None
        self._coeffs, self._scales = np.asarray(coeffs, dtype=np.float64), np.ones(len(coeffs))
        return self

    def save_params(self, filename: str = "polymlp_params.yaml"):
        from pypolymlp_gb300.features_attr import write_polymlp_params_yaml

        if self._params is None:
            raise RuntimeError("Set parameters first.")
        write_polymlp_params_yaml(self._params, filename)
        return self

    def save_errors(self, filename: str = "polymlp_error.yaml"):
        """Errors in the layout of eval_accuracy.py:271-301 (meV/atom, eV/angstrom)."""
        if self._error_train is None:
            raise RuntimeError("estimate_error must be performed before save_errors.")
        with open(filename, "w") as f:
            print("units:\n  energy: meV/atom\n  force:  eV/angstrom\n  stress: meV/atom\n", file=f)
            print("prediction_errors:", file=f)
            for errors in (self._error_train, self._error_test):
                for key, e in errors.items():
                    print("- dataset:", key, file=f)
                    print("  rmse_energy: ", e["energy"] * 1000, file=f)
                    if e["force"] is not None:
                        print("  rmse_force:  ", e["force"], file=f)
                    if e["stress"] is not None:
                        print("  rmse_stress: ", e["stress"] * 1000, file=f)
                    print("", file=f)
                    print("  mae_energy:  ", e["energy_mae"] * 1000, file=f)
                    if e["force_mae"] is not None:
                        print("  mae_force:   ", e["force_mae"], file=f)
                    if e["stress_mae"] is not None:
                        print("  mae_stress:  ", e["stress_mae"] * 1000, file=f)
                    print("", file=f)
        return self

    # -- results --------------------------------------------------------------------
    @property
    def parameters(self) -> dict:
        return self._params

    @property
    def coeffs(self):
        """Coefficients of the unscaled features (c / s)."""
        return None if self._coeffs is None else self._coeffs / self._scales

    @property
    def n_features(self) -> int:
        from pypolymlp_gb300.features_attr import get_num_features

        return get_num_features(self._models)

    @property
    def errors(self):
        return self._error_train, self._error_test

    @property
    def learning_curve(self):
        return self._learning_log

    @property
    def train(self):
        return self._train

    @property
    def test(self):
        return self._test

    @property
    def fit_result(self):
        return self._result
