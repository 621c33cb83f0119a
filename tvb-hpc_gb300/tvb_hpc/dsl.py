"""
The CUDA DSL's launcher interface (dsl/dsl_cuda/example/cuda_run.py and
cuda_setup.py) on the engine: a model named by its LEMS file runs as the
engine's generated kernels instead of a pycuda-compiled template.

    from tvb_hpc.dsl import CudaRun, expand_params, setup_params
    couplings, speeds = setup_params(32, 32)            # cuda_setup.py:97-101
    params = expand_params(couplings, speeds)          # cuda_setup.py:88-94
    tavg = CudaRun().run_simulation(weights, lengths, params, speeds, logger, args,
                                    n_nodes, n_work_items, n_params, nstep,
                                    n_inner_steps, buf_len, states, dt, min_speed)

`args` needs `model` (the LEMS model name, e.g. 'Kuramoto') and may carry
`lems_folder` (default: the bundled model files).  The return value is the
reference's tavg layout, (nstep, n_nodes * n_exposures, n_work_items): the
exposures after each launch of n_inner_steps steps.  (The reference appends
the host buffer before copying each launch's result into it,
cuda_run.py:138-142, so its first row is zeros and its last launch is
dropped; here row i is the result of launch i.)  buf_len (the history
length) is planned by the engine from the delays, and min_speed is not
needed: the delays come from each work item's global_speed.
"""

import itertools

import numpy as np

from . import lems


def setup_params(nc, ns):
    "couplings logspace(1.6, 3.0, nc), speeds logspace(0, 2, ns) (cuda_setup.py:97-101)."
    return np.logspace(1.6, 3.0, nc), np.logspace(0.0, 2.0, ns)


def expand_params(couplings, speeds):
    "Work items (speed, coupling) in itertools.product order, float32 (cuda_setup.py:88-94)."
    return np.array(list(itertools.product(speeds, couplings)), np.float32)


class CudaRun:
    "cuda_run.CudaRun on the engine (the model comes from its LEMS file)."

    def run_simulation(self, weights, lengths, params_matrix, speeds, logger, args, n_nodes,
                       n_work_items, n_params, nstep, n_inner_steps, buf_len, states, dt,
                       min_speed):
        m = lems.load_model(args.model, getattr(args, 'lems_folder', None))
        params = np.asarray(params_matrix, np.float32).reshape(n_work_items, n_params)
        if n_params != len(m.params):
            raise ValueError('%s takes %d swept parameters, got %d'
                             % (m.name, len(m.params), n_params))
        if states != m.ns:
            raise ValueError('%s has %d state variables, got states=%d' % (m.name, m.ns, states))
        w = np.asarray(weights, np.float32).reshape(n_nodes, n_nodes)
        ln = np.asarray(lengths, np.float32).reshape(n_nodes, n_nodes)
        if logger is not None:
            logger.info('engine: %s, %d work items x %d nodes, %d launches of %d steps'
                        % (m.name, n_work_items, n_nodes, nstep, n_inner_steps))
        tavg, self.sweep = lems.run_simulation(m, w, ln, params, dt, nstep, n_inner_steps)
        return tavg
