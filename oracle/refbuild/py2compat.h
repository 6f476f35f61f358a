/* Python-2 C-API names used by the reference module, mapped onto Python 3.
 *
 * TEST INFRASTRUCTURE ONLY.  This header is force-included (gcc -include)
 * ahead of the unmodified cmod/src/centmodule.c so that the reference's own
 * source compiles against a Python 3 interpreter; no line of the reference
 * file is edited.  The reference uses (cmod/src/centmodule.c):
 *   PyInt_AsLong / PyInt_Check       :2590-2826, :3022-3023
 *   Py_InitModule("cent", methods)    :3327 (inside initcent, :3323)
 * Python 3 has no separate int type (PyLong is the int) and creates modules
 * from a PyModuleDef; refcompat_init_module() (pyinit.c) does that and keeps
 * the module for PyInit_cent to return.
 */
#ifndef DASP_REF_PY2COMPAT_H
#define DASP_REF_PY2COMPAT_H

#include <Python.h>

#define PyInt_AsLong PyLong_AsLong
#define PyInt_Check PyLong_Check
#define PyInt_FromLong PyLong_FromLong

PyObject *refcompat_init_module(const char *name, PyMethodDef *methods);
#define Py_InitModule(name, methods) refcompat_init_module((name), (methods))

#endif
