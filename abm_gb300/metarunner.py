"""Batched front-end of the reference's metarunner (abm/metarunner/metarunner.py).

The reference sweeps parameters by writing one .env file per combination and running the
simulations one after another (MetaProtocol.generate_temp_env_files / run_protocols,
metarunner.py:167-254).  ``BatchedProtocol`` takes the same sweep definitions — ``Constant``,
``Tunable`` (values = np.linspace(min, max, n) or an explicit list), ``TunedPairRestrain``
(add_tuned_pair: the product of two values must equal a constant; add_quadratic_tuned_pair:
value1 * value2**2 must be close to it), ``num_batches`` repetitions — expands them into the
same list of configurations in the same order (itertools.product over the criteria in the
order they were added, then the restraints, then one copy per batch), and runs the
visual-flocking configurations as batched launches: configurations that differ only in
parameters the batched step takes per agent (VF_ALP0, VF_BET0, VF_V0, RADIUS_AGENT, and the
agent count N) share one abm_vpf_flock_batched launch sequence; every other difference starts
another group.  Agents start like VFSimulation.create_agents (vf_sims.py:212-227: headings
uniform, positions on a disc around the arena centre, facing out), from numpy's generator
seeded per configuration.
"""
from __future__ import annotations

import itertools
from typing import Optional

import numpy as np

from .params import VFParams


class Tunable:
    """A parameter to sweep (metarunner.py:59-91): np.linspace(min_v, max_v, num_data_points)
    including both ends, or the given values_override (which wins when both are given)."""

    def __init__(self, var_name, min_v=None, max_v=None, num_data_points=None,
                 values_override=None):
        if min_v is None and values_override is None:
            raise ValueError("Neither value borders nor override values have been given to "
                             "create Tunable!")
        self.name = var_name
        if values_override is None:
            self.values = np.linspace(min_v, max_v, num=num_data_points, endpoint=True)
        else:
            self.values = values_override

    def get_values(self):
        return self.values


class Constant:
    """One fixed value (metarunner.py:30-42)."""

    def __init__(self, var_name, constant):
        self.tunable = Tunable(var_name, values_override=[constant])
        self.name = self.tunable.name

    def get_values(self):
        return self.tunable.values


class TunedPairRestrain:
    """Two parameters whose product is restrained (metarunner.py:44-56)."""

    def __init__(self, var_name1, var_name2, restrained_product):
        self.var1, self.var2 = var_name1, var_name2
        self.product_restrain = restrained_product

    def get_vars(self):
        return [self.var1, self.var2]


# parameters the batched step accepts per agent (abm_agent_overrides) or per instance (N)
PER_AGENT_KEYS = ("VF_ALP0", "VF_BET0", "VF_V0", "RADIUS_AGENT", "N")


class BatchedProtocol:
    """MetaProtocol's sweep definition, run as batched launches."""

    def __init__(self, base_env: dict, num_batches: int = 1, experiment_name: Optional[str] = None):
        self.base_env = dict(base_env)
        self.num_batches = int(num_batches)
        self.experiment_name = experiment_name
        self.tunables, self.tuned_pairs, self.q_tuned_pairs = [], [], []

    def add_criterion(self, criterion):
        self.tunables.append(criterion)

    def add_tuned_pair(self, pair):
        self.tuned_pairs.append(pair)

    def add_quadratic_tuned_pair(self, pair):
        self.q_tuned_pairs.append(pair)

    # ------------------------------------------------------------------ expansion
    def combos(self):
        """The value combinations the reference keeps (generate_temp_env_files +
        consider_tuned_pairs, metarunner.py:136-189): exact product test for tuned pairs,
        np.isclose for quadratic ones; a combination failing several restraints is removed
        once."""
        names = [t.name for t in self.tunables]
        combos = list(itertools.product(*[t.get_values() for t in self.tunables]))
        kept = combos.copy()
        for pair in self.tuned_pairs:
            for combo in combos:
                product = 1
                for j, value in enumerate(combo):
                    if names[j] in pair.get_vars():
                        product *= value
                if product != pair.product_restrain and combo in kept:
                    kept.remove(combo)
        for pair in self.q_tuned_pairs:
            for combo in combos:
                product = 1
                for j, value in enumerate(combo):
                    if names[j] == pair.get_vars()[0]:
                        product *= value
                    elif names[j] == pair.get_vars()[1]:
                        product *= value * value
                if not np.isclose(product, pair.product_restrain) and combo in kept:
                    kept.remove(combo)
        return kept

    def env_configs(self):
        """One .env mapping per run, in the reference's generation order (batch nb outer,
        combination i inner; the file {i}_b{nb}.env): the base file with the combination's
        values (booleans as 0/1) and SAVE_ROOT_DIR of that batch."""
        names = [t.name for t in self.tunables]
        out = []
        for nb in range(self.num_batches):
            for combo in self.combos():
                env = dict(self.base_env)
                for name, value in zip(names, combo):
                    env[name] = int(value) if isinstance(value, bool) else value
                exp = self.experiment_name if self.experiment_name is not None else "UnknownExp"
                env["SAVE_ROOT_DIR"] = f"abm/data/simulation_data/{exp}/batch_{nb}"
                out.append(env)
        return out

    def env_files(self):
        """(file name, .env mapping) in the order the reference runs them: run_protocols
        (metarunner.py:240-254) takes the files {i}_b{nb}.env sorted by name."""
        combos = len(self.combos())
        named = [(f"{i}_b{nb}.env", env) for idx, env in enumerate(self.env_configs())
                 for nb, i in [divmod(idx, combos)]]
        return sorted(named, key=lambda t: t[0])

    # ------------------------------------------------------------------ batched runs
    @staticmethod
    def _group_key(env):
        p = VFParams.from_env(env)
        return (p.gam, p.alp1, p.alp2, p.bet1, p.bet2, p.boundary, p.limit_movement,
                p.max_vel, p.max_th, p.width, p.height, p.window_pad, tuple(p.fov), p.rv,
                p.dt)

    def groups(self):
        """Configuration indices grouped by everything the batched step cannot vary."""
        order, groups = [], {}
        for idx, env in enumerate(self.env_configs()):
            key = self._group_key(env)
            if key not in groups:
                groups[key] = []
                order.append(key)
            groups[key].append(idx)
        return [groups[k] for k in order]

    @staticmethod
    def initial_state(env, seed):
        """VFSimulation.create_agents (vf_sims.py:212-227) with numpy's generator."""
        p = VFParams.from_env(env)
        n = int(float(env.get("N", 10)))
        rng = np.random.default_rng(seed)
        ori = rng.uniform(0, 2 * np.pi, n)
        dist = rng.random(n) * (p.height / 2 - 2 * p.window_pad - p.radius)
        x = np.cos(ori) * dist + p.width / 2
        y = np.sin(ori) * dist + p.height / 2
        return {"x": x.astype(np.float32), "y": y.astype(np.float32),
                "theta": ori.astype(np.float32), "v": np.zeros(n, np.float32)}

    def instances(self, seed=0):
        """(params, instance dict) per configuration, in configuration order; the instance
        carries its ALP0 / BET0 and, where they differ from the first configuration of its
        group, its V0 and radius as per-agent values."""
        envs = self.env_configs()
        first = {}
        for members in self.groups():
            for m in members:
                first[m] = VFParams.from_env(envs[members[0]])
        out = []
        for idx, env in enumerate(envs):
            p = VFParams.from_env(env)
            inst = self.initial_state(env, seed + idx)
            inst.update(alp0=p.alp0, bet0=p.bet0)
            if p.v0 != first[idx].v0:
                inst["v0"] = p.v0
            if p.radius != first[idx].radius:
                inst["radius"] = p.radius
            out.append((p, inst))
        return out

    def run_folders(self, save_root: str):
        """Where run() writes each configuration's data: save_root/<its SAVE_ROOT_DIR>/<the
        stem of its .env file name>, in configuration order (the reference writes a run into
        a time-stamped folder under SAVE_ROOT_DIR, ifdb_params.py:33-39; its ExperimentLoader
        takes every folder of a batch, data_loader.py:459-466)."""
        import os
        combos = len(self.combos())
        out = []
        for idx, env in enumerate(self.env_configs()):
            nb, i = divmod(idx, combos)
            out.append(os.path.join(save_root, env["SAVE_ROOT_DIR"], f"{i}_b{nb}"))
        return out

    def run(self, steps: int, seed: int = 0, chunk: int = 100, device="cuda",
            save_root: Optional[str] = None, as_zarr: Optional[bool] = None,
            save_extracted_vfield: bool = False):
        """Run every configuration for `steps` steps, one BatchedSweep per group; returns the
        final state of each configuration (dicts of numpy arrays) in configuration order.

        save_root: also record every step on the device and write each configuration's run as
        the reference writes one simulation's data at its end (vf_sims.py:373-381: the JSON
        files, or the zarr arrays when as_zarr — by default the configuration's
        USE_ZARR_FORMAT —, and env_params.json with the values as its .env file holds them)
        into the folders of run_folders(save_root)."""
        from .batched import BatchedSweep
        insts = self.instances(seed)
        envs = self.env_configs()
        folders = self.run_folders(save_root) if save_root is not None else None

        def zarr_of(env):
            if as_zarr is not None:
                return bool(as_zarr)
            return bool(int(float(env.get("USE_ZARR_FORMAT", 0))))

        results = [None] * len(insts)
        for members in self.groups():
            base = insts[members[0]][0]
            sweep = BatchedSweep(base, [insts[m][1] for m in members], device=device)
            if folders is not None:
                vpf = save_extracted_vfield or not all(zarr_of(envs[m]) for m in members)
                sweep.record_steps(steps, vpf=vpf)
            if steps >= chunk:
                sweep.run(steps, chunk=chunk)
            else:
                for _ in range(steps):
                    sweep.step()
            for k, m in enumerate(members):
                results[m] = sweep.instance_state(k)
                if folders is not None:
                    env_json = {key: f"{val}" for key, val in envs[m].items()}
                    sweep.save_reference_run(k, folders[m], zarr_of(envs[m]), env_json,
                                             save_extracted_vfield)
        return results
