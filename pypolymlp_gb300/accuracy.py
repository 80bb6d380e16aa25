"""Prediction errors of a fitted potential on datasets, evaluated on the GPU.

`PolymlpEvalAccuracy` mirrors the reference's class of the same name
(src/pypolymlp/mlp_dev/core/eval_accuracy.py:16-149): `compute_error` runs
`compute_error_single` over datasets; per dataset the E/F/S predictions come
from the GPU evaluator (`pg_eval_run`, through `PotentialPropertiesFast`) and
the errors are
  energy  RMSE and MAE of energies per atom (eV/atom),
  force   RMSE and MAE over all force components (eV/angstrom), optionally
          the mean relative error of the force norms and the angle (degrees)
          of the mean |cosine| between true and predicted force directions,
  stress  RMSE and MAE of the six components per structure, per atom (eV) or
          in GPa (eV per cell / volume x 160.21766208),
as eval_accuracy.py:60-133 computes them; `prediction_errors` is that
arithmetic on given predictions (numpy, no device).  With log_* set the true
and predicted values are written to <path_output>/predictions/ like
eval_accuracy.py:216-270 (structures named by their index: the datasets here
carry no file names).
"""

from __future__ import annotations

import os
from math import acos, degrees
from typing import Literal, Optional, Sequence

import numpy as np

EV_TO_GPA = 160.21766208


def _rmse(t, p):
    return float(np.sqrt(np.mean(np.square(t - p))))


def _mae(t, p):
    return float(np.mean(np.abs(t - p)))


def prediction_errors(dataset, energies, forces, stresses, stress_unit: Literal["eV", "GPa"] = "eV",
                      force_direction: bool = False):
    """Error dictionary of predictions (energies (n_st,), forces: list of
    (N, 3), stresses (n_st, 6)) against a dataset, plus the (true, predicted)
    arrays used: {"energy", "force", "stress", "energy_mae", "force_mae",
    "stress_mae", "percent_force_norm", "force_direction"}, arrays."""
    n_atoms = np.asarray(dataset.total_n_atoms, dtype=np.float64)
    true_e = np.asarray(dataset.energies, dtype=np.float64) / n_atoms
    pred_e = np.asarray(energies, dtype=np.float64) / n_atoms
    err = {"energy": _rmse(true_e, pred_e), "energy_mae": _mae(true_e, pred_e), "force": None, "force_mae": None,
           "stress": None, "stress_mae": None, "percent_force_norm": None, "force_direction": None}
    arrays = {"energy": (true_e, pred_e)}
    # errors wherever the data exist, fitted or not (eval_accuracy.py:82, 115: exist_force / exist_stress)
    if dataset.forces is not None:
        true_f = np.concatenate([np.asarray(f, dtype=np.float64).reshape(-1) for f in dataset.forces])
        pred_f = np.concatenate([np.asarray(f, dtype=np.float64).reshape(-1) for f in forces])
        err["force"], err["force_mae"] = _rmse(true_f, pred_f), _mae(true_f, pred_f)
        arrays["force"] = (true_f, pred_f)
        if force_direction:
            t3, p3 = true_f.reshape(-1, 3), pred_f.reshape(-1, 3)
            nt, npred = np.linalg.norm(t3, axis=1), np.linalg.norm(p3, axis=1)
            cosine = np.einsum("ij,ij->i", t3 / nt[:, None], p3 / npred[:, None])
            err["percent_force_norm"] = float(np.average(np.abs((npred - nt) / nt)))
            err["force_direction"] = degrees(acos(min(1.0, float(np.average(np.abs(cosine))))))
    if dataset.stresses is not None:
        if stress_unit == "eV":
            norm = np.repeat(n_atoms, 6)
        elif stress_unit == "GPa":
            vol = np.array([abs(np.linalg.det(np.asarray(a, dtype=np.float64))) for a in dataset.axis])
            norm = np.repeat(vol, 6) / EV_TO_GPA
        else:
            raise ValueError("stress_unit must be 'eV' or 'GPa'")
        true_s = np.asarray(dataset.stresses, dtype=np.float64).reshape(-1) / norm
        pred_s = np.asarray(stresses, dtype=np.float64).reshape(-1) / norm
        err["stress"], err["stress_mae"] = _rmse(true_s, pred_s), _mae(true_s, pred_s)
        arrays["stress"] = (true_s, pred_s)
    return err, arrays


class PolymlpEvalAccuracy:
    """Errors of the potential (params dict, coefficients already divided by
    the feature scales) on datasets (`regression.Dataset`)."""

    def __init__(self, params_dict: dict, scaled_coeffs, precision: Optional[int] = None, verbose: bool = False):
        from pypolymlp_gb300 import _ffi
        from pypolymlp_gb300.properties import PotentialPropertiesFast

        self._prop = PotentialPropertiesFast(params_dict, scaled_coeffs,
                                             _ffi.PG_FP64 if precision is None else precision)
        self._verbose = verbose

    def compute_error(self, datasets: Sequence, stress_unit: Literal["eV", "GPa"] = "eV", log_energy: bool = True,
                      log_force: bool = False, log_stress: bool = False, path_output: str = "./",
                      tag: str = "train"):
        return {d.name: self.compute_error_single(d, output_key=self._output_key(d.name, tag), stress_unit=stress_unit,
                                                  log_energy=log_energy, log_force=log_force, log_stress=log_stress,
                                                  path_output=path_output)
                for d in datasets}

    def compute_error_single(self, dataset, output_key: str = "train", stress_unit: Literal["eV", "GPa"] = "eV",
                             log_energy: bool = True, log_force: bool = False, log_stress: bool = False,
                             path_output: str = "./", force_direction: bool = False):
        self._prop.eval_multiple(dataset.axis, [np.asarray(p, dtype=np.float64).T for p in dataset.positions],
                                 dataset.types)
        err, arrays = prediction_errors(dataset, self._prop.get_e_array(), self._prop.get_f_array(),
                                        self._prop.get_s_array(), stress_unit, force_direction)
        if self._verbose:
            self.print_error(err, key=output_key)
        logs = [(log_energy, "energy", "# DFT(eV/atom), MLP(eV/atom), DFT-MLP(meV/atom)", 1000.0),
                (log_force, "force", "# DFT, MLP, DFT-MLP", 1.0), (log_stress, "stress", "# DFT, MLP, DFT-MLP", 1.0)]
        for on, name, header, scale in logs:
            if not on or name not in arrays:
                continue
            os.makedirs(os.path.join(path_output, "predictions"), exist_ok=True)
            t, p = arrays[name]
            with open(os.path.join(path_output, "predictions", f"{name}.{output_key}.dat"), "w") as f:
                print(header, file=f)
                for q, (a, b) in enumerate(zip(t, p)):
                    print(a, b, (a - b) * scale, *([f"structure-{q}"] if name == "energy" else []), file=f)
        return err

    @staticmethod
    def print_error(error: dict, key: str = "train"):
        print("prediction:", key, flush=True)
        print("  rmse_energy:", "{0:13.5f}".format(error["energy"] * 1000), "(meV/atom)", flush=True)
        if error["force"] is not None:
            print("  rmse_force: ", "{0:13.5f}".format(error["force"]), "(eV/ang)", flush=True)
        if error["stress"] is not None:
            print("  rmse_stress:", "{0:13.5f}".format(error["stress"] * 1000), "(meV/atom)", flush=True)
        print("  mae_energy: ", "{0:13.5f}".format(error["energy_mae"] * 1000), "(meV/atom)", flush=True)
        if error["force_mae"] is not None:
            print("  mae_force:  ", "{0:13.5f}".format(error["force_mae"]), "(eV/ang)", flush=True)
        if error["stress_mae"] is not None:
            print("  mae_stress: ", "{0:13.5f}".format(error["stress_mae"] * 1000), "(meV/atom)", flush=True)

    @staticmethod
    def _output_key(dataset_name: str, tag: str) -> str:
        key = dataset_name.replace("*", "-").replace("." + "./", "")
        key = tag + "-" + key.replace(".", "-").replace("/", "-")
        return key.replace("---", "-").replace("--", "-")
