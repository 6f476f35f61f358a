/* Python 3 module entry for the reference's ``cent`` module -- TEST
 * INFRASTRUCTURE ONLY.
 *
 * The reference registers its methods in a Python-2 style ``initcent``
 * (cmod/src/centmodule.c:3323-3331: Py_InitModule("cent", centMethods),
 * import_array, the cent.error exception).  Python 3 looks for PyInit_cent
 * and expects the module object back; this file supplies both halves:
 * refcompat_init_module() builds the module from a PyModuleDef when
 * initcent calls Py_InitModule (mapped in py2compat.h), and PyInit_cent
 * runs initcent and returns that module.
 */
#include <Python.h>

void initcent(void);

static PyObject *g_module = NULL;
static struct PyModuleDef g_def;

PyObject *refcompat_init_module(const char *name, PyMethodDef *methods) {
    struct PyModuleDef head = {PyModuleDef_HEAD_INIT};
    g_def = head;
    g_def.m_name = name;
    g_def.m_doc = "DASP centmodule (reference build, Python 3 shim)";
    g_def.m_size = -1;
    g_def.m_methods = methods;
    g_module = PyModule_Create(&g_def);
    return g_module;
}

PyMODINIT_FUNC PyInit_cent(void) {
    g_module = NULL;
    initcent();
    if (PyErr_Occurred()) {
        Py_XDECREF(g_module);
        return NULL;
    }
    return g_module;
}
