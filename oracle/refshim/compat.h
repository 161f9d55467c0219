/* Forced-include header for compiling the MAPP sources against Python 3.12
 * and NumPy 2 (test infrastructure only).  Included before every reference
 * translation unit with `-include`:
 *  - Python 3.12 made Py_TYPE and Py_REFCNT inline functions, so the
 *    reference's `Py_TYPE(x) = type` and `Py_REFCNT(x) = 1` assignments
 *    need the old lvalue macros back;
 *  - Python 3.11 folded co_varnames into co_localsplusnames, whose first
 *    co_argcount entries are still the argument names the reference reads;
 *  - NumPy 2 exposes PyArray_Descr::elsize only to 2.x-API builds
 *    (NPY_TARGET_VERSION is set on the command line).
 */
#ifndef MAPPG_REF_COMPAT_H
#define MAPPG_REF_COMPAT_H
#ifdef __cplusplus
#include <Python.h>
#undef Py_TYPE
#define Py_TYPE(ob) (((PyObject*)(ob))->ob_type)
#undef Py_REFCNT
#define Py_REFCNT(ob) (((PyObject*)(ob))->ob_refcnt)
#define co_varnames co_localsplusnames
#endif
#endif
