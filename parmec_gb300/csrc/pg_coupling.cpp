// pg_coupling.cpp -- the C library interface of parmec (parmec.h:291-310) over
// the package's commands (parmec_gb300/coupling.py), declared in
// include/parmec_coupling.h.
//
// The reference's libparmec8 embeds CPython to read decks (input.cpp) and
// runs the DEM loop in C++.  Here the deck commands and the DEM driver live
// in the Python package and the step runs on the GPU session, so this
// library embeds the interpreter (or joins the calling process's) and calls
// the package.  Every call takes the GIL for its duration.
#include <Python.h>
#include <dlfcn.h>
#include <cstdio>
#include <cstring>
#include <string>
#include "../../include/parmec_coupling.h"

namespace {

PyObject *g_mod = nullptr;

// the repository root: two directories above this library (parmec_gb300/_build/)
std::string repo_root()
{
  Dl_info info;
  if (!dladdr((void *)&repo_root, &info) || !info.dli_fname) return std::string();
  std::string p(info.dli_fname);
  for (int up = 0; up < 3; up ++)
  {
    const size_t k = p.rfind('/');
    if (k == std::string::npos) return std::string();
    p = p.substr(0, k);
  }
  return p;
}

struct Gil
{
  PyGILState_STATE st;
  Gil() : st(PyGILState_Ensure()) {}
  ~Gil() { PyGILState_Release(st); }
};

bool ready()
{
  if (!Py_IsInitialized())
  {
    Py_InitializeEx(0);
    // the embedding thread holds the GIL after initialisation; release it so
    // that every call takes it the same way
    PyEval_SaveThread();
  }
  if (g_mod) return true;
  Gil gil;
  const std::string root = repo_root();
  PyObject *sys_path = PySys_GetObject("path");                 // borrowed
  if (sys_path && !root.empty())
  {
    PyObject *r = PyUnicode_FromString(root.c_str());
    if (r) { PyList_Insert(sys_path, 0, r); Py_DECREF(r); }
  }
  g_mod = PyImport_ImportModule("parmec_gb300.coupling");
  if (!g_mod) { PyErr_Print(); return false; }
  return true;
}

// call coupling.<name>(*args); returns a new reference or null (error printed)
PyObject *call(const char *name, PyObject *args)
{
  PyObject *fn = PyObject_GetAttrString(g_mod, name);
  PyObject *res = fn ? PyObject_CallObject(fn, args) : nullptr;
  Py_XDECREF(fn);
  Py_XDECREF(args);
  if (!res) PyErr_Print();
  return res;
}

int int_result(PyObject *r)
{
  if (!r) return -1;
  const long v = PyLong_Check(r) ? PyLong_AsLong(r) : 0;
  Py_DECREF(r);
  return (int)v;
}

PyObject *triple(const double *v)
{
  return v ? Py_BuildValue("(ddd)", v[0], v[1], v[2]) : (Py_INCREF(Py_None), Py_None);
}

} // namespace

extern "C" {

int pg_parmec_init(void)
{
  if (!ready()) return -1;
  Gil gil;
  return int_result(call("init", PyTuple_New(0)));
}

int pg_parmec_reset(void)
{
  if (!ready()) return -1;
  Gil gil;
  return int_result(call("reset", PyTuple_New(0)));
}

int pg_parmec_input(const char *path, char **argv, int argc)
{
  if (!path || argc < 0 || !ready()) return -1;
  Gil gil;
  PyObject *lst = PyList_New(0);
  for (int k = 0; k < argc; k ++)
  {
    PyObject *a = PyUnicode_FromString(argv[k] ? argv[k] : "");
    PyList_Append(lst, a);
    Py_DECREF(a);
  }
  return int_result(call("input", Py_BuildValue("(sN)", path, lst)));
}

double pg_parmec_dem(double duration, double step, const double *interval, const char *prefix, int verbose,
                     double adaptive)
{
  if (!ready()) return -1.0;
  Gil gil;
  PyObject *iv = interval ? Py_BuildValue("(dd)", interval[0], interval[1]) : (Py_INCREF(Py_None), Py_None);
  PyObject *pf = prefix ? PyUnicode_FromString(prefix) : (Py_INCREF(Py_None), Py_None);
  PyObject *r = call("dem", Py_BuildValue("(ddNNid)", duration, step, iv, pf, verbose, adaptive));
  if (!r) return -1.0;
  const double v = PyFloat_AsDouble(r);
  Py_DECREF(r);
  return v;
}

int pg_parmec_declare_analytical(int k)
{
  if (!ready()) return -1;
  Gil gil;
  return int_result(call("declare_analytical", Py_BuildValue("(i)", k)));
}

int pg_parmec_set_body_force(int k, const double outer_force[3], const double outer_torque[3])
{
  if (!ready()) return -1;
  Gil gil;
  const double zero[3] = {0.0, 0.0, 0.0};
  PyObject *f = triple(outer_force);
  PyObject *t = triple(outer_force ? (outer_torque ? outer_torque : zero) : nullptr);
  return int_result(call("set_body_force", Py_BuildValue("(iNN)", k, f, t)));
}

int pg_parmec_get_body_force(int k, double inner_force[3], double inner_torque[3])
{
  if (!ready()) return -1;
  Gil gil;
  PyObject *r = call("get_body_force", Py_BuildValue("(i)", k));
  if (!r) return -1;
  if (r == Py_None) { Py_DECREF(r); return -1; }
  double v[6];
  for (int c = 0; c < 6; c ++) v[c] = PyFloat_AsDouble(PyTuple_GetItem(r, c));
  Py_DECREF(r);
  for (int c = 0; c < 3; c ++)
  {
    if (inner_force) inner_force[c] = v[c];
    if (inner_torque) inner_torque[c] = v[3 + c];
  }
  return 0;
}

int pg_parmec_parnum(void)
{
  if (!ready()) return -1;
  Gil gil;
  return int_result(call("parnum", PyTuple_New(0)));
}

int pg_parmec_particle(int k, double position[3], double linear[3], double angular[3])
{
  if (!ready()) return -1;
  Gil gil;
  PyObject *r = call("particle", Py_BuildValue("(i)", k));
  if (!r) return -1;
  double v[9];
  for (int c = 0; c < 9; c ++) v[c] = PyFloat_AsDouble(PyTuple_GetItem(r, c));
  Py_DECREF(r);
  for (int c = 0; c < 3; c ++)
  {
    if (position) position[c] = v[c];
    if (linear) linear[c] = v[3 + c];
    if (angular) angular[c] = v[6 + c];
  }
  return 0;
}

} // extern "C"
