"""The MCMC caller: likelihood objects as sampler models.

Mirror of dust2's `dust_likelihood_monty` (R/monty.R:90-253): a model
whose density at a parameter vector is the log-likelihood of a filter or
unfilter run at the unpacked parameters, with the generator hand-off a
stochastic model needs (R/monty.R:212-224: the sampler hands over one
32-byte stream state, expanded to the object's streams by jumps, as
`filter_rng_state` does, R/interface-filter.R:120-124) and an observer
of the last state and trajectories (R/monty.R:286-317).

`served_model` is the same density through the likelihood server, so
that many chains, each in its own thread, evaluate on one device at once
(the server is reached through the C ABI, dust2_gb300_server_*).
`random_walk` is a small random-walk Metropolis sampler used to drive
such chains (monty's sampler is an R package; this one follows the
standard algorithm: propose x' = x + L z with z ~ N(0, I), accept with
probability min(1, exp(d(x') - d(x))).
"""

import threading

import numpy as np

from ._lib import DustError
from .interface import (DustLikelihood, DustUnfilter,
                        dust_likelihood_last_gradient,
                        dust_likelihood_last_state,
                        dust_likelihood_last_trajectories,
                        dust_likelihood_rng_state, dust_likelihood_run,
                        dust_likelihood_set_rng_state, rng_streams)


class Packer:
    """A packer for scalar parameters (monty_packer with scalars only):
    `names` are the sampled parameters in vector order, `fixed` holds
    values that are not sampled."""

    def __init__(self, names, fixed=None):
        self._names = list(names)
        if len(set(self._names)) != len(self._names):
            raise DustError("Parameter names must be unique")
        self.fixed = dict(fixed or {})
        clash = set(self._names) & set(self.fixed)
        if clash:
            raise DustError(f"Parameters both sampled and fixed: "
                            f"{sorted(clash)}")

    def names(self):
        return list(self._names)

    def unpack(self, x):
        x = np.asarray(x, dtype=float).ravel()
        if x.size != len(self._names):
            raise DustError(f"Expected a parameter vector of length "
                            f"{len(self._names)}, but it had {x.size}")
        ret = dict(self.fixed)
        ret.update({nm: float(v) for nm, v in zip(self._names, x)})
        return ret

    def pack(self, pars):
        return np.array([float(pars[nm]) for nm in self._names])


class DustModel:
    """A sampler model: density(x), and for stochastic likelihoods the
    generator hand-off; `observe()` returns the observer's record."""

    def __init__(self, parameters, density, properties, get_rng_state=None,
                 set_rng_state=None, observer=None, likelihood=None,
                 gradient=None):
        self.parameters = parameters
        self.density = density
        self.gradient = gradient
        self.properties = properties
        self.get_rng_state = get_rng_state
        self.set_rng_state = set_rng_state
        self.observer = observer
        self.likelihood = likelihood

    def observe(self):
        if self.observer is None:
            raise DustError("This model has no observer")
        return self.observer()


def _n_streams(obj):
    npg = getattr(obj, "n_particles_per_group", None)
    if npg is not None:
        return sum(n + 2 for n in npg)
    return max(1, obj.n_groups) * (obj.n_particles + 2)


def dust_likelihood_monty(obj, packer, initial=None,
                          failure_is_impossible=False, save_state=False,
                          save_trajectories=False):
    """R/monty.R:90-253 for a filter (stochastic) or unfilter
    (deterministic) object with one parameter group."""
    if not isinstance(obj, (DustLikelihood, DustUnfilter)):
        raise DustError("Expected 'obj' to be a 'dust_likelihood' object")
    if obj.n_groups != 1:
        raise DustError("Models over several parameter groups need a "
                        "grouped packer, which this mirror does not have")
    deterministic = isinstance(obj, DustUnfilter)
    cache = {}

    def run(x):
        pars = packer.unpack(x)
        init = None if initial is None else initial(pars)
        ll = dust_likelihood_run(obj, pars, initial=init,
                                 save_trajectories=bool(save_trajectories))
        return float(np.sum(ll))

    has_gradient = deterministic and obj.generator.has_adjoint
    gradient = None
    if deterministic:
        def density(x):
            key = np.asarray(x, dtype=float).tobytes()
            if cache.get("key") != key:
                cache["value"] = run(x)
                cache["key"] = key
                cache.pop("gradient", None)
            return cache["value"]

        if has_gradient:
            # R/monty.R:176-185: the gradient at x of the last adjoint run
            # (the density runs with the adjoint by default), kept with the
            # density until x changes
            def gradient(x):
                density(x)
                if "gradient" not in cache:
                    cache["gradient"] = np.ravel(
                        dust_likelihood_last_gradient(obj))
                return cache["gradient"]
    else:
        density = run

    if failure_is_impossible:
        inner = density

        def density(x):  # noqa: F811 (R/monty.R:197-199, protect())
            try:
                return inner(x)
            except DustError:
                return -np.inf

    observer = None
    if save_state or save_trajectories:
        def observer():
            ret = {}
            if save_state:
                ret["state"] = dust_likelihood_last_state(
                    obj, select_random_particle=True)
            if save_trajectories:
                ret["trajectories"] = dust_likelihood_last_trajectories(
                    obj, select_random_particle=True)
            return ret

    get_rng_state = set_rng_state = None
    if not deterministic:
        def get_rng_state():
            return dust_likelihood_rng_state(obj)

        def set_rng_state(state):
            # the sampler hands over one stream (32 bytes); the others
            # follow by jumps (R/monty.R:216-223)
            dust_likelihood_set_rng_state(
                obj, rng_streams(_n_streams(obj), bytes(state)[:32]))

    properties = {"is_stochastic": not deterministic,
                  "has_direct_sample": False, "has_gradient": has_gradient,
                  "allow_multiple_parameters": False,
                  "has_observer": observer is not None,
                  "has_parameter_groups": False}
    return DustModel(packer.names(), density, properties, get_rng_state,
                     set_rng_state, observer, obj, gradient)


def served_model(server, session, packer, failure_is_impossible=False):
    """The density of one server session (a one-group filter likelihood)
    as a sampler model; each call submits a request and waits for it, so
    chains in separate threads overlap on the device."""
    def density(x):
        pars = packer.unpack(x)
        try:
            return server.likelihood(session, pars)
        except DustError:
            if failure_is_impossible:
                return -np.inf
            raise

    properties = {"is_stochastic": True, "has_direct_sample": False,
                  "has_gradient": False, "allow_multiple_parameters": False,
                  "has_observer": False, "has_parameter_groups": False}
    return DustModel(packer.names(), density, properties)


def random_walk(model, vcv, n_steps, initial, seed=0, prior=None):
    """Random-walk Metropolis for one chain: proposal N(x, vcv); the
    target is density(x) + prior(x) (prior returns a log density, default
    flat).  Returns (samples [n_steps][n_pars], log densities, acceptance
    rate)."""
    rs = np.random.default_rng(seed)
    chol = np.linalg.cholesky(np.atleast_2d(np.asarray(vcv, dtype=float)))
    x = np.asarray(initial, dtype=float).copy()

    def target(v):
        lp = 0.0 if prior is None else float(prior(v))
        if not np.isfinite(lp):
            return -np.inf
        return lp + model.density(v)

    d = target(x)
    out = np.empty((n_steps, x.size))
    dens = np.empty(n_steps)
    accepted = 0
    for i in range(n_steps):
        prop = x + chol @ rs.standard_normal(x.size)
        dp = target(prop)
        if np.log(rs.uniform()) < dp - d:
            x, d = prop, dp
            accepted += 1
        out[i] = x
        dens[i] = d
    return out, dens, accepted / n_steps


def run_chains(models, vcv, n_steps, initial, seed=0, prior=None):
    """One random-walk chain per model, each in its own thread (for
    served models the chains' requests share the device); results in
    model order."""
    res = [None] * len(models)
    errors = []

    def go(i):
        try:
            res[i] = random_walk(models[i], vcv, n_steps, initial[i],
                                 seed=seed + i, prior=prior)
        except Exception as e:  # noqa: BLE001 - reported below
            errors.append(e)

    threads = [threading.Thread(target=go, args=(i,))
               for i in range(len(models))]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    if errors:
        raise errors[0]
    return res
