"""ctypes binding of include/rajzel_io.h and a writer of RAJZEL parameter
directories in the reference's file formats, for the I/O and driver tests."""
import ctypes as C
import os

import numpy as np

PATH = 256
_INT, _F, _S = C.c_int, C.c_float, C.c_char * PATH


class Par(C.Structure):
    _fields_ = [("INVMAT", _INT), ("NX", _INT), ("NY", _INT), ("DH", _F), ("TIME", _F), ("SOURCE_FILE", _S),
                ("READMOD", _INT), ("MFILE", _S), ("SNAP", _INT), ("IDX", _INT), ("IDY", _INT),
                ("SNAP_FORMAT", _INT), ("SNAP_FILE", _S), ("SEISMO", _INT), ("REC_FILE", _S),
                ("REFREC", _F * 2), ("N_STREAMER", _INT), ("REC_INCR_X", _F), ("REC_INCR_Y", _F),
                ("PICKS_FILE", _S), ("TTNORM", _F), ("LOG_FILE", _S), ("LOG", _INT), ("ITERMAX", _INT),
                ("EPS_ADJ", _F), ("JACOBIAN", _S), ("DATA_DIR", _S), ("TAPER", _INT), ("TAPERLENGTH", _INT),
                ("INVTYPE", _INT), ("GRADT1", _INT), ("GRADT2", _INT), ("GRADT3", _INT), ("GRADT4", _INT),
                ("SWS_TAPER_GRAD_VERT", _INT), ("SWS_TAPER_GRAD_HOR", _INT), ("EXP_TAPER_GRAD_HOR", _F),
                ("SWS_TAPER_GRAD_SOURCES", _INT), ("SWS_TAPER_CIRCULAR_PER_SHOT", _INT), ("SRTSHAPE", _INT),
                ("SRTRADIUS", _F), ("FILTSIZE", _INT), ("SWS_TAPER_FILE", _INT), ("INV_MODELFILE", _S),
                ("nfstart", _INT), ("nf", _INT), ("nfstart_jac", _INT), ("nf_jac", _INT), ("VPUPPERLIM", _F),
                ("VPLOWERLIM", _F), ("GRAD_METHOD", _INT), ("NLBFGS", _INT), ("MODEL_FILTER", _INT),
                ("FILT_SIZE", _INT), ("LINESEARCH", _INT), ("EPS_SCALE", _F), ("C1", _F), ("C2", _F),
                ("STEPMAX", _INT), ("SCALEFAC", _F), ("MISFIT_LOG_FILE", _S), ("MIN_ITER", _INT),
                ("GRAD_FILTER", _INT), ("FILT_SIZE_GRAD", _INT), ("VP0_1", _F), ("VP0_2", _F), ("DVP0", _F),
                ("GRAD0_1", _F), ("GRAD0_2", _F), ("DGRAD0", _F), ("GRIDSEARCH_FILE", _S), ("nlines", _INT)]


def lib():
    from rajzel_gb300 import build as B
    B.build()
    L = C.CDLL(B.LIB)
    L.rz_io_error.restype = C.c_char_p
    return L


# one "label = value" line per parameter, in the reference's order (read_par.c)
ORDER = ["INVMAT", "NX", "NY", "DH", "TIME", "SOURCE_FILE", "READMOD", "MFILE", "SNAP", "IDX", "IDY", "SNAP_FORMAT",
         "SNAP_FILE", "SEISMO", "REC_FILE", "REFREC", "N_STREAMER", "REC_INCR_X", "REC_INCR_Y", "PICKS_FILE",
         "TTNORM", "LOG_FILE", "LOG", "ITERMAX", "EPS_ADJ", "JACOBIAN", "DATA_DIR", "TAPER", "TAPERLENGTH",
         "INVTYPE", "GRADT", "SWS_TAPER_GRAD_VERT", "SWS_TAPER_GRAD_HOR", "EXP_TAPER_GRAD_HOR",
         "SWS_TAPER_GRAD_SOURCES", "SWS_TAPER_CIRCULAR_PER_SHOT", "SRTSHAPE", "SRTRADIUS", "FILTSIZE",
         "SWS_TAPER_FILE", "INV_MODELFILE", "nfstart", "nf", "nfstart_jac", "nf_jac", "VPUPPERLIM", "VPLOWERLIM",
         "GRAD_METHOD", "NLBFGS", "MODEL_FILTER", "FILT_SIZE", "LINESEARCH", "EPS_SCALE", "C1C2", "STEPMAX",
         "SCALEFAC", "MISFIT_LOG_FILE", "MIN_ITER", "GRAD_FILTER", "FILT_SIZE_GRAD", "VP0", "GRAD0",
         "GRIDSEARCH_FILE"]

DEFAULTS = dict(INVMAT=0, SNAP=0, IDX=1, IDY=1, SNAP_FORMAT=3, SNAP_FILE="tt/snap", SEISMO=1, REFREC="0.0 , 0.0",
                N_STREAMER=0, REC_INCR_X=0.0, REC_INCR_Y=0.0, PICKS_FILE="picks/picks", TTNORM=1e-6,
                LOG_FILE="log/rz.log", LOG=1, ITERMAX=3, EPS_ADJ=1e-9, JACOBIAN="grad/grad", DATA_DIR="obs/picks",
                TAPER=0, TAPERLENGTH=4, INVTYPE=2, GRADT="3, 5, 90, 100", SWS_TAPER_GRAD_VERT=0,
                SWS_TAPER_GRAD_HOR=0, EXP_TAPER_GRAD_HOR=0.0, SWS_TAPER_GRAD_SOURCES=0,
                SWS_TAPER_CIRCULAR_PER_SHOT=0, SRTSHAPE=1, SRTRADIUS=80.0, FILTSIZE=1, SWS_TAPER_FILE=0,
                INV_MODELFILE="model/inv", nfstart=2000, nf=2000, nfstart_jac=2000, nf_jac=1, VPUPPERLIM=6000.0,
                VPLOWERLIM=1000.0, GRAD_METHOD=2, NLBFGS=5, MODEL_FILTER=0, FILT_SIZE=5, LINESEARCH=1,
                EPS_SCALE=0.01, C1C2="1e-4, 0.9", STEPMAX=10, SCALEFAC=2.0, MISFIT_LOG_FILE="misfit.dat",
                MIN_ITER=0, GRAD_FILTER=0, FILT_SIZE_GRAD=0, VP0="1500.0, 1700.0, 100.0",
                GRAD0="0.5, 1.5, 0.5", GRIDSEARCH_FILE="grid.dat", READMOD=1, MFILE="model/true")


def write_inp(path, **kw):
    v = dict(DEFAULTS, **kw)
    lines = ["#-------------------------------------------", "# parameter file written by the tests", "#"]
    for i, k in enumerate(ORDER):
        if i % 7 == 3:
            lines.append("# a comment line between parameters")
        lines.append(f"{k} = {v[k]}")
    with open(path, "w") as f:
        f.write("\n".join(lines) + "\n")


def write_sources(path, xs, zs):
    with open(path, "w") as f:
        f.write(f"{len(xs)} \n")
        for x, z in zip(xs, zs):
            f.write(f"{x:.2f} \t 0.00 \t {z:.2f} \t 0.00 \t 10.00 \t 1.00 \t 0.00 \t 1 \n")


def write_receivers(path, xs, zs):
    with open(path, "w") as f:
        for x, z in zip(xs, zs):
            f.write(f"{x:.3f}\t{z:.3f}\n")


def write_model(path, vp):
    """writemod.c format 3: float32, x outer."""
    np.ascontiguousarray(np.asarray(vp, np.float32).T).tofile(path)


def read_model(path, nx, ny):
    return np.fromfile(path, np.float32).reshape(nx, ny).T


def read_picks(prefix, shot):
    return np.array([float(x) for x in open(f"{prefix}_{shot}.dat").read().split()], np.float32)


def write_picks(prefix, shot, t):
    with open(f"{prefix}_{shot}.dat", "w") as f:
        for v in t:
            f.write("%e \n" % v)


def makedirs(root, *names):
    for n in names:
        os.makedirs(os.path.join(root, n), exist_ok=True)
