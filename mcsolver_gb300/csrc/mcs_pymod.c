/*
 * mcs_pymod.c -- CPython extension modules isinglib / xylib / heisenberglib,
 * drop-in replacements for mcsolver's compiled libraries.
 *
 * Compiled three times, with -DMCS_PYMOD=1 (isinglib), 2 (xylib) or
 * 3 (heisenberglib).  Each module exports one METH_VARARGS function
 * MCMainFunction with the reference's positional arguments:
 *   isinglib       isingLib.c:277-284      16 arguments, returns the 11-tuple of isingLib.c:436-447
 *   xylib          xyLib.c:439-447         23 arguments, returns the 29-tuple of xyLib.c:778-807
 *   heisenberglib  heisenbergLib.c:504-512 23 arguments, returns the 29-tuple of heisenbergLib.c:853-884
 * and forwards to mcs_solve() of libmcsgpu.so with the GIL released.
 *
 * Differences from the reference, all on the error path: arguments are
 * validated (ValueError for malformed input, RuntimeError with the engine's
 * message for device errors) instead of being read unchecked, and every
 * buffer is released.  Engine knobs the signature cannot carry come from the
 * environment: MCSGPU_SEED (Philox key, default 1 -- the reference's unseeded
 * rand() also starts every process from seed 1), MCSGPU_SCHEDULE
 * (auto|plain|resident|tiled), MCSGPU_ABSOLUTE_ENERGY=1, MCSGPU_DEVICE.
 */
#define PY_SSIZE_T_CLEAN
#include <Python.h>
#include <stdlib.h>
#include <string.h>

#include "../../include/mcsgpu.h"

#ifndef MCS_PYMOD
#error "define MCS_PYMOD to 1 (Ising), 2 (XY) or 3 (Heisenberg)"
#endif

#if MCS_PYMOD == 1
#define MODNAME "isinglib"
#define INITFN PyInit_isinglib
#define NARGS 16
#elif MCS_PYMOD == 2
#define MODNAME "xylib"
#define INITFN PyInit_xylib
#define NARGS 23
#else
#define MODNAME "heisenberglib"
#define INITFN PyInit_heisenberglib
#define NARGS 23
#endif

typedef struct {
    double *d;
    int32_t *i;
    Py_ssize_t n;
} Arr;

static int to_doubles(PyObject *o, Arr *a, const char *name)
{
    PyObject *f = PySequence_Fast(o, name);
    if (!f) return -1;
    Py_ssize_t n = PySequence_Fast_GET_SIZE(f);
    a->n = n;
    a->d = (double *)malloc(sizeof(double) * (n > 0 ? n : 1));
    if (!a->d) { Py_DECREF(f); PyErr_NoMemory(); return -1; }
    PyObject **it = PySequence_Fast_ITEMS(f);
    for (Py_ssize_t k = 0; k < n; ++k) {
        double v = PyFloat_AsDouble(it[k]);
        if (v == -1.0 && PyErr_Occurred()) { Py_DECREF(f); return -1; }
        a->d[k] = v;
    }
    Py_DECREF(f);
    return 0;
}

static int to_ints(PyObject *o, Arr *a, const char *name)
{
    PyObject *f = PySequence_Fast(o, name);
    if (!f) return -1;
    Py_ssize_t n = PySequence_Fast_GET_SIZE(f);
    a->n = n;
    a->i = (int32_t *)malloc(sizeof(int32_t) * (n > 0 ? n : 1));
    if (!a->i) { Py_DECREF(f); PyErr_NoMemory(); return -1; }
    PyObject **it = PySequence_Fast_ITEMS(f);
    for (Py_ssize_t k = 0; k < n; ++k) {
        long v = PyLong_AsLong(it[k]);
        if (v == -1 && PyErr_Occurred()) { Py_DECREF(f); return -1; }
        if (v < INT32_MIN || v > INT32_MAX) { Py_DECREF(f); PyErr_Format(PyExc_ValueError, "%s: value out of range", name); return -1; }
        a->i[k] = (int32_t)v;
    }
    Py_DECREF(f);
    return 0;
}

static int to_long(PyObject *o, long long *v, const char *name)
{
    *v = PyLong_AsLongLong(o);
    if (*v == -1 && PyErr_Occurred()) {
        PyErr_Format(PyExc_TypeError, "%s must be an integer", name);
        return -1;
    }
    return 0;
}

static void options_from_env(mcs_options *o)
{
    memset(o, 0, sizeof *o);
    const char *s = getenv("MCSGPU_SEED");
    o->seed = s ? strtoull(s, NULL, 0) : 1ULL;
    s = getenv("MCSGPU_SCHEDULE");
    if (s) {
        if (!strcmp(s, "plain")) o->schedule = 1;
        else if (!strcmp(s, "resident")) o->schedule = 2;
        else if (!strcmp(s, "tiled")) o->schedule = 3;
    }
    s = getenv("MCSGPU_ABSOLUTE_ENERGY");
    o->absolute_energy = (s && atoi(s)) ? 1 : 0;
    s = getenv("MCSGPU_DEVICE");
    o->device = s ? atoi(s) : 0;
}

static PyObject *MCMainFunction(PyObject *self, PyObject *args)
{
    (void)self;
    if (!PyTuple_Check(args) || PyTuple_GET_SIZE(args) != NARGS) {
        PyErr_Format(PyExc_TypeError, "MCMainFunction expects %d positional arguments", NARGS);
        return NULL;
    }
    PyObject *a[NARGS];
    for (int k = 0; k < NARGS; ++k) a[k] = PyTuple_GET_ITEM(args, k);
    mcs_problem p;
    memset(&p, 0, sizeof p);
    Arr init = {0}, initD = {0}, nlink = {0}, ls = {0}, lo = {0}, circ = {0}, cp = {0}, glist = {0};
    Arr rorb = {0}, rcl = {0}, rlink = {0};
    long long alg, nth, nsw, tau, z, frames, ngroup = 0, maxg = 1, ign = 0;
    double flunc = 0.0, h;
    PyObject *ret = NULL;
    float *fbuf = NULL;
    double *gbuf = NULL;
#if MCS_PYMOD == 1
    /* isingLib.c:277-284 */
    if (to_long(a[0], &alg, "algorithm") || to_doubles(a[1], &init, "initSpin") || to_long(a[2], &nth, "nthermal") ||
        to_long(a[3], &nsw, "nsweep") || to_long(a[4], &tau, "ninterval") || to_long(a[5], &z, "maxNLinking") ||
        to_ints(a[6], &nlink, "nlink") || to_doubles(a[7], &ls, "linkStrength") || to_ints(a[8], &lo, "linkedOrb") ||
        to_ints(a[9], &cp, "corrOrbPair"))
        goto done;
    h = PyFloat_AsDouble(a[10]);
    if (h == -1.0 && PyErr_Occurred()) goto done;
    if (to_ints(a[11], &rorb, "rOrb") || to_ints(a[12], &rcl, "rOrbCluster") || to_ints(a[13], &rlink, "linkedOrb_rnorm") ||
        to_long(a[14], &frames, "spinFrame"))
        goto done;
    p.model = MCS_ISING;
#else
    /* heisenbergLib.c:504-512 / xyLib.c:439-447 */
    if (to_long(a[0], &alg, "algorithm") || to_doubles(a[1], &init, "initSpin") || to_doubles(a[2], &initD, "initD") ||
        to_long(a[3], &nth, "nthermal") || to_long(a[4], &nsw, "nsweep") || to_long(a[5], &tau, "ninterval") ||
        to_long(a[6], &z, "maxNLinking") || to_ints(a[7], &nlink, "nlink") || to_doubles(a[8], &ls, "linkStrength") ||
        to_ints(a[9], &lo, "linkedOrb") || to_ints(a[10], &circ, "localCircuits") || to_ints(a[11], &cp, "corrOrbPair") ||
        to_long(a[12], &ngroup, "nOrbGroup") || to_long(a[13], &maxg, "maxOrbGroupSize") || to_ints(a[14], &glist, "orbGroupList"))
        goto done;
    flunc = PyFloat_AsDouble(a[15]);
    if (flunc == -1.0 && PyErr_Occurred()) goto done;
    h = PyFloat_AsDouble(a[16]);
    if (h == -1.0 && PyErr_Occurred()) goto done;
    if (to_ints(a[17], &rorb, "rOrb") || to_ints(a[18], &rcl, "rOrbCluster") || to_ints(a[19], &rlink, "linkedOrb_rnorm") ||
        to_long(a[20], &frames, "spinFrame") || to_long(a[21], &ign, "ignoreNonDiagonalJ"))
        goto done;
    p.model = MCS_PYMOD == 2 ? MCS_XY : MCS_HEISENBERG;
#endif
    {
        Py_ssize_t N = init.n;
        if (N <= 0) { PyErr_SetString(PyExc_ValueError, "initSpin is empty"); goto done; }
        if (z < 0 || z > 32) { PyErr_SetString(PyExc_ValueError, "maxNLinking out of range"); goto done; }
        Py_ssize_t per = (p.model == MCS_ISING) ? 1 : 9;
        if (nlink.n != N || lo.n != N * z || ls.n != N * z * per) {
            PyErr_SetString(PyExc_ValueError, "nlink / linkedOrb / linkStrength sizes do not match initSpin and maxNLinking");
            goto done;
        }
        if (p.model != MCS_ISING && initD.n != 3 * N) { PyErr_SetString(PyExc_ValueError, "initD must hold 3 values per site"); goto done; }
        if (cp.n < 2 || (cp.n & 1)) { PyErr_SetString(PyExc_ValueError, "corrOrbPair must hold pairs"); goto done; }
        if (rorb.n < 1 || rcl.n < rorb.n || rcl.n % rorb.n) { PyErr_SetString(PyExc_ValueError, "rOrb / rOrbCluster sizes inconsistent"); goto done; }
        if (rlink.n != rorb.n * z) { PyErr_SetString(PyExc_ValueError, "linkedOrb_rnorm size must be len(rOrb)*maxNLinking"); goto done; }
        if (circ.n % 3) { PyErr_SetString(PyExc_ValueError, "localCircuits must hold triples"); goto done; }
        if (ngroup < 0 || maxg < 0 || glist.n < ngroup * maxg) { PyErr_SetString(PyExc_ValueError, "orbGroupList too short"); goto done; }
        p.algorithm = (int32_t)alg;
        p.n_sites = (int32_t)N;
        p.max_links = (int32_t)z;
        p.nthermal = nth; p.nsweep = nsw; p.ninterval = tau;
        p.init_spin = init.d;
        p.init_d = initD.d;
        p.nlink = nlink.i;
        p.link_strength = ls.d;
        p.linked_orb = lo.i;
        p.circuits = circ.i; p.n_circuits = (int32_t)(circ.n / 3);
        p.corr_pair = cp.i; p.n_lat = (int32_t)(cp.n / 2);
        p.group_list = glist.i; p.n_group = (int32_t)ngroup; p.max_group = (int32_t)maxg;
        p.r_orb = rorb.i; p.n_rorb = (int32_t)rorb.n;
        p.r_cluster = rcl.i; p.n_in_cluster = (int32_t)(rcl.n / rorb.n);
        p.r_link = rlink.i;
        p.flunc = flunc; p.h = h;
        p.ignore_offdiag = (int32_t)ign;
        if (frames < 0 || frames > nsw) { PyErr_SetString(PyExc_ValueError, "spinFrame must be in [0, nsweep]"); goto done; }
        p.spin_frames = (int32_t)frames;

        mcs_options o;
        options_from_env(&o);
        mcs_result r;
        memset(&r, 0, sizeof r);
        int G = (p.model == MCS_ISING) ? 0 : (int)ngroup;
        int ng = (G + 1) * (G + 1) + (G + 1);
        gbuf = (double *)calloc((size_t)ng, sizeof(double));
        if (!gbuf) { PyErr_NoMemory(); goto done; }
        r.group_values = gbuf;
        r.group_capacity = ng;
        if (frames > 0) {
            fbuf = (float *)malloc(sizeof(float) * 3 * (size_t)N * (size_t)frames);
            if (!fbuf) { PyErr_NoMemory(); goto done; }
            r.frames = fbuf;
        }
        int rc;
        Py_BEGIN_ALLOW_THREADS
        rc = mcs_solve(&p, &o, &r);
        Py_END_ALLOW_THREADS
        if (rc != MCS_OK) {
            PyErr_Format((rc == MCS_EINVAL || rc == MCS_EUNSUPPORTED) ? PyExc_ValueError : PyExc_RuntimeError,
                         "mcsgpu error %d: %s", rc, mcs_last_error());
            goto done;
        }
        /* spin frames: tuple of frames, each a tuple over sites (isingLib.c:381-386,
           heisenbergLib.c:664-675); a float 0.0 when no frames were asked for */
        PyObject *frameobj;
        if (frames > 0) {
            frameobj = PyTuple_New(frames);
            if (!frameobj) goto done;
            for (long long f = 0; f < frames; ++f) {
                if (f >= r.frames_written) { Py_INCREF(Py_None); PyTuple_SET_ITEM(frameobj, f, Py_None); continue; }
                PyObject *fr = PyTuple_New(N);
                if (!fr) { Py_DECREF(frameobj); goto done; }
                PyTuple_SET_ITEM(frameobj, f, fr);
                for (Py_ssize_t i = 0; i < N; ++i) {
                    const float *q = fbuf + ((size_t)f * N + i) * 3;
                    PyObject *v = (p.model == MCS_ISING)
                                      ? PyFloat_FromDouble(q[0])
                                      : Py_BuildValue("(ddd)", (double)q[0], (double)q[1], (double)q[2]);
                    if (!v) { Py_DECREF(frameobj); goto done; }
                    PyTuple_SET_ITEM(fr, i, v);
                }
            }
        } else {
            frameobj = PyFloat_FromDouble(0.0);
            if (!frameobj) goto done;
        }
#if MCS_PYMOD == 1
        ret = PyTuple_New(11);
        if (!ret) { Py_DECREF(frameobj); goto done; }
        PyTuple_SET_ITEM(ret, 10, frameobj);
        for (int k = 0; k < 10; ++k) {
            PyObject *v = PyFloat_FromDouble(r.values[k]);
            if (!v) { Py_CLEAR(ret); goto done; }
            PyTuple_SET_ITEM(ret, k, v);
        }
#else
        ret = PyTuple_New(29);
        if (!ret) { Py_DECREF(frameobj); goto done; }
        PyTuple_SET_ITEM(ret, 27, frameobj);
        for (int k = 0; k < 27; ++k) {
            PyObject *v = PyFloat_FromDouble(r.values[k]);
            if (!v) { Py_CLEAR(ret); goto done; }
            PyTuple_SET_ITEM(ret, k, v);
        }
        PyObject *gt;
        if (G > 0) {
            gt = PyTuple_New(ng);
            if (!gt) { Py_CLEAR(ret); goto done; }
            PyTuple_SET_ITEM(ret, 28, gt);
            for (int k = 0; k < ng; ++k) {
                PyObject *v = PyFloat_FromDouble(gbuf[k]);
                if (!v) { Py_CLEAR(ret); goto done; }
                PyTuple_SET_ITEM(gt, k, v);
            }
        } else {
            gt = PyFloat_FromDouble(0.0);
            if (!gt) { Py_CLEAR(ret); goto done; }
            PyTuple_SET_ITEM(ret, 28, gt);
        }
#endif
    }
done:
    free(init.d); free(initD.d); free(nlink.i); free(ls.d); free(lo.i); free(circ.i); free(cp.i); free(glist.i);
    free(rorb.i); free(rcl.i); free(rlink.i); free(fbuf); free(gbuf);
    return ret;
}

static PyMethodDef methods[] = {
    {"MCMainFunction", MCMainFunction, METH_VARARGS, "Monte Carlo solve of one (T,H) point on the GPU"},
    {NULL, NULL, 0, NULL}};

static struct PyModuleDef moddef = {PyModuleDef_HEAD_INIT, MODNAME,
                                    "GB300 drop-in for mcsolver's " MODNAME " (MCMainFunction)", -1, methods};

PyMODINIT_FUNC INITFN(void) { return PyModule_Create(&moddef); }
