"""Drop-in for tdscha.StaticHessian (Modules/StaticHessian.py) on the GPU.

The unknown is the vector [G (upper triangle rows, M(M+1)/2) | W (i <= j <= k,
M(M+1)(M+2)/6)]; one application of the system matrix applies the static
operator to the M rows [G_i | W_i] (StaticHessian.apply_L, :561-620).  Here the
vector lives in device memory, the M rows are formed and collected by
tdscha_static_hessian_expand / _collect and the M static applications run as
one batched tdscha_static_L call; the minimal-residual iteration
(Tools.minimum_residual_algorithm / _precond) runs on device tensors.
"""
import difflib
import json
import os
import sys
import time

import numpy as np

from . import _native as nat
from . import Tools
from .DynamicalLanczos import Lanczos, TYPE_DP, _torch


class StaticHessian(object):
    def __init__(self, ensemble=None, verbose=False, lanczos_input={}):
        self.vector = None
        self.lanczos_input = lanczos_input
        self.lanczos = Lanczos(ensemble, **lanczos_input)
        self.verbose = False
        self.prefix = "hessian_calculation"
        self.preconitioned = True
        if ensemble is not None:
            self.init(ensemble, verbose)
        self.__total_attributes__ = [item for item in self.__dict__.keys()]
        self.fixed_attributes = True

    def __setattr__(self, name, value):
        """Unknown attributes raise, with close matches suggested (:70-88)."""
        if "fixed_attributes" in self.__dict__:
            if name in self.__total_attributes__:
                super(StaticHessian, self).__setattr__(name, value)
            elif self.fixed_attributes:
                similar = str(difflib.get_close_matches(name, self.__total_attributes__))
                raise AttributeError("\n        Error, the attribute '{}' is not a member of '{}'.\n"
                                     "        Suggested similar attributes: {} ?\n        "
                                     .format(name, type(self).__name__, similar))
        else:
            super(StaticHessian, self).__setattr__(name, value)

    # --------------------------------------------------------------- sizes
    def _sizes(self):
        M = self.lanczos.n_modes
        return M, (M * (M + 1)) // 2, (M * (M ** 2 + 3 * M + 2)) // 6

    def _initial_vector(self):
        M, n_g, n_w = self._sizes()
        v = np.zeros(n_g + n_w, dtype=TYPE_DP)
        counter = 0
        for i in range(M):
            v[counter] = 1 / self.lanczos.w[i] if self.preconitioned else 1 / self.lanczos.w[i] ** 2
            counter += M - i
        return v

    def init(self, ensemble=None, verbose=True):
        """Set up the Lanczos object and the initial guess (the SSCHA matrix,
        :133-181).  Without an ensemble, a Lanczos object already holding data
        (e.g. Lanczos.from_arrays, assigned to .lanczos) is used."""
        if ensemble is not None:
            self.lanczos = Lanczos(ensemble, **self.lanczos_input)
            self.lanczos.init()
            self.vector = self._initial_vector()
        else:
            if self.lanczos.N == 0:
                raise ValueError("Error, you must specify an ensemble or initialize the system "
                                 "loading a lanczos algorithm.")
            if not self.lanczos.initialized:
                self.lanczos.init()
            if self.vector is None:
                self.vector = self._initial_vector()
        self.verbose = verbose
        if verbose:
            print("Memory of StaticHessian initialized.")
            print("     memory requested: {} Gb of RAM per process".format(
                self.vector.nbytes * 3 / 1024 ** 3))
            print("     (excluding memory occupied to store the ensemble)")

    # ------------------------------------------------------------ operator
    def _apply_dev(self, v, preconditioner=False, inverse_preconditioner=False):
        """System matrix on a device vector (one batched static application)."""
        torch = _torch()
        if preconditioner and inverse_preconditioner:
            raise ValueError("Error, only one between preconditioner and inverse_preconditioner "
                             "can be True")
        lz = self.lanczos
        ctx = lz._context()
        M = lz.n_modes
        Ps = lz._static_size()
        st = torch.cuda.current_stream().cuda_stream
        lib = nat.load()
        X = torch.empty((M, Ps), dtype=torch.float64, device=v.device)
        nat.check(lib.tdscha_static_hessian_expand(ctx.handle, v.data_ptr(), X.data_ptr(), st))
        if preconditioner:
            Y = lz._static_dev(X, 1, -0.5)
        elif inverse_preconditioner:
            Y = lz._static_dev(X, 1, 0.5)
        else:
            Y = lz._static_dev(X, 3)
        out = torch.empty_like(v)
        nat.check(lib.tdscha_static_hessian_collect(ctx.handle, Y.data_ptr(), out.data_ptr(), st))
        return out

    def apply_L(self, vect, preconditioner=False, inverse_preconditioner=False):
        """Apply the system matrix to the full vector (:561-620), numpy in and out."""
        torch = _torch()
        v = torch.from_numpy(np.ascontiguousarray(vect, dtype=np.float64)).cuda()
        out = self._apply_dev(v, preconditioner, inverse_preconditioner)
        nat.check(nat.load().tdscha_ctx_sync(self.lanczos._ctx.handle,
                                             torch.cuda.current_stream().cuda_stream))
        return out.cpu().numpy()

    def run(self, n_steps, save_dir=None, threshold=1e-6, algorithm="cg-prec", extra_options={}):
        """Solve for G and W (:184-286) with the minimal-residual iteration
        ('cg') or its preconditioned form ('cg-prec'), on the GPU."""
        torch = _torch()
        if save_dir is not None and not os.path.exists(save_dir):
            os.makedirs(save_dir)
        M, n_g, n_w = self._sizes()
        lenv = len(self.vector)
        dev = torch.device("cuda")

        class _Op:
            def __init__(op, **kw):
                op.kw = kw

            def matvec(op, x):
                return self._apply_dev(x, **op.kw)

        A = _Op()
        A_precond_half = _Op(preconditioner=True)

        def callback(x, iters):
            if save_dir is not None:
                np.savetxt(os.path.join(save_dir, "{}_step{:05d}.dat".format(self.prefix, iters)),
                           x.cpu().numpy())
            sys.stdout.flush()

        x0 = torch.from_numpy(self.vector.copy()).to(dev)
        b = torch.zeros(lenv, dtype=torch.float64, device=dev)
        counter = 0
        for i in range(M):
            b[counter] = 1
            counter += M - i
        t1 = time.time()
        if algorithm.lower() == "cg":
            res = Tools.minimum_residual_algorithm(A, b, x0, max_iters=n_steps,
                                                   conv_thr=threshold, callback=callback,
                                                   verbose=self.verbose)
        elif algorithm.lower() == "cg-prec":
            res = Tools.minimum_residual_algorithm_precond(A, b, A_precond_half, x0=x0,
                                                           max_iters=n_steps, conv_thr=threshold,
                                                           callback=callback,
                                                           verbose=self.verbose)
        else:
            raise NotImplementedError("Error, algorithm '{}' not implemented.".format(algorithm))
        nat.check(nat.load().tdscha_ctx_sync(self.lanczos._ctx.handle,
                                             torch.cuda.current_stream().cuda_stream))
        t2 = time.time()
        self.vector[:] = res.cpu().numpy()
        if save_dir is not None:
            self.save_status(os.path.join(save_dir, self.prefix))
        if self.verbose:
            print()
            print("HESSIAN CALCULATION CONVERGED")
            print("Total time to converge: {:.2f} s".format(t2 - t1))
            print()

    def run_no_mode_mixing(self, nsteps, save_dir=None, restart_from_file=False, noq=False):
        """Hessian without mode mixing (:403-496): one Lanczos run per mode of the
        auxiliary force constants (prepare_mode, run_FT on the GPU), G_ii = Re G(0) of
        its continued fraction without terminator, W = 0.  A mode degenerate with the
        one before it (|w_i - w_{i-1}| < 1e-10) is not run again and takes that run's
        G(0).  save_dir keeps each run's steps and final status
        (<prefix>_M<i>_conv), from which restart_from_file resumes.  Returns
        retrieve_hessian(noq)."""
        lanc = self.lanczos
        M = lanc.n_modes
        Gw = np.zeros((M, M), dtype=np.double)
        if save_dir is not None and not os.path.exists(save_dir):
            os.makedirs(save_dir)
        for i in range(M):
            if i > 0 and np.abs(lanc.w[i - 1] - lanc.w[i]) < 1e-10:
                if self.verbose:
                    print("SKIPPING MODE {} (Degeneracy)".format(i + 1))
            else:
                lanc.prepare_mode(i)
                if self.verbose:
                    head = "RUNNING MODE {} out of {}".format(i + 1, M)
                    print("\n" + head + "\n" + "-" * len(head) + "\n")
                todo = nsteps
                tag = self.prefix + "_M{:d}".format(i + 1)
                final = None if save_dir is None else os.path.join(save_dir, tag + "_conv")
                if save_dir is not None and restart_from_file:
                    self._resume_mode(final, save_dir, tag)
                    if len(lanc.a_coeffs):
                        todo = nsteps - len(lanc.a_coeffs)
                if todo > 0:
                    lanc.run_FT(todo, save_dir=save_dir, verbose=self.verbose, prefix=tag)
                if final is not None:
                    lanc.save_status(final)
            gf0 = lanc.get_green_function_continued_fraction(np.array([0]), use_terminator=False,
                                                             smearing=0)[0]
            Gw[i, i] = np.real(gf0)
        W = np.zeros((M, M, M), dtype=np.double)
        self.preconitioned = False
        self.vector = self.get_vector(Gw, W)
        return self.retrieve_hessian(noq=noq)

    def _resume_mode(self, final, save_dir, tag):
        """Load a mode's final status, else its latest <tag>_STEP<n>.npz (:463-480).
        The final status is looked up with its .npz suffix and the step files by
        "<tag>_STEP", so that mode 1 does not pick up the files of modes 10-19."""
        lanc = self.lanczos
        for name in (final, final + ".npz"):
            if os.path.exists(name):
                if self.verbose:
                    print("Loading from {}...".format(name))
                lanc.load_status(name)
                return
        steps = [x for x in os.listdir(save_dir)
                 if x.startswith(tag + "_STEP") and x.endswith(".npz")]
        if steps:
            count = [int(x.split(".")[-2].split("STEP")[-1]) for x in steps]
            name = os.path.join(save_dir, steps[int(np.argmax(count))])
            if self.verbose:
                print("Loading from {}...".format(name))
            lanc.load_status(name)

    # ------------------------------------------------------------- layout
    def get_G_W(self, vector, ignore_W=False):
        """G (symmetric) and W (fully symmetric) from the vector (:625-658)."""
        M, n_g, n_w = self._sizes()
        vector = np.asarray(vector)
        G = np.zeros((M, M), dtype=np.double)
        iu = np.triu_indices(M)
        G[iu] = vector[:n_g]
        G.T[iu] = vector[:n_g]
        if ignore_W:
            return G
        i, j, k = _upper3(M)
        W = np.zeros((M, M, M), dtype=np.double)
        vals = vector[n_g:n_g + n_w]
        for a, b, c in ((i, j, k), (i, k, j), (j, i, k), (j, k, i), (k, i, j), (k, j, i)):
            W[a, b, c] = vals
        return G, W

    def get_vector(self, G, W):
        """Upper parts of G and W as the vector (:660-691)."""
        M, n_g, n_w = self._sizes()
        iu = np.triu_indices(M)
        i, j, k = _upper3(M)
        return np.concatenate([np.asarray(G)[iu], np.asarray(W)[i, j, k]]).astype(np.double)

    def retrieve_hessian(self, noq=False):
        """The Hessian from the solved vector (:510-558); noq=True returns the
        supercell matrix pols G^-1 pols^T scaled by sqrt(m_a m_b)."""
        new_vector = self.vector.copy()
        if self.preconitioned:
            new_vector = self.apply_L(self.vector, preconditioner=True)
        Ginv = self.get_G_W(new_vector, ignore_W=True)
        G = np.linalg.inv(Ginv)
        dyn = self.lanczos.pols.dot(G.dot(self.lanczos.pols.T))
        dyn[:, :] *= np.outer(np.sqrt(self.lanczos.m), np.sqrt(self.lanczos.m))
        if noq:
            return dyn
        try:
            import cellconstructor as CC
            import cellconstructor.Phonons
        except ImportError as e:
            raise ImportError("retrieve_hessian(noq=False) builds a CC.Phonons object and needs "
                              "cellconstructor; use noq=True for the supercell matrix") from e
        nq_tot = len(self.lanczos.dyn.q_tot)
        q_points = np.array(self.lanczos.dyn.q_tot)
        uc = self.lanczos.dyn.structure.copy()
        ss = self.lanczos.dyn.structure.generate_supercell(self.lanczos.dyn.GetSupercell())
        dynq = CC.Phonons.GetDynQFromFCSupercell(dyn, q_points, uc, ss)
        hessian = CC.Phonons.Phonons(self.lanczos.dyn.structure, nqirr=nq_tot)
        for i in range(nq_tot):
            hessian.dynmats[i] = dynq[i, :, :]
            hessian.q_tot[i] = q_points[i, :]
        hessian.AdjustQStar()
        return hessian

    # ---------------------------------------------------------------- I/O
    def save_status(self, fname):
        np.savetxt(fname, self.vector)
        self.lanczos.save_status(fname)
        skip = ["lanczos", "vector", "fixed_attributes", "__total_attributes__"]
        with open(fname + ".json", "w") as fp:
            json.dump({k: v for k, v in vars(self).items() if k not in skip}, fp)

    def load_status(self, fname):
        self.lanczos.load_status(fname + ".npz")
        self.lanczos.init(use_symmetries=False)
        self.vector = np.loadtxt(fname)
        with open(fname + ".json", "r") as fp:
            for k, v in json.load(fp).items():
                self.__setattr__(k, v)


def _upper3(M):
    """(i, j, k) with i <= j <= k in the order of the vector's W part."""
    i, j, k = [], [], []
    for a in range(M):
        jj, kk = np.triu_indices(M - a)
        i.append(np.full(len(jj), a))
        j.append(jj + a)
        k.append(kk + a)
    return np.concatenate(i), np.concatenate(j), np.concatenate(k)
