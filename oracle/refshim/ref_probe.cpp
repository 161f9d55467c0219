/* Probe entry points linked into the reference module built from the MAPP
 * sources (oracle/_ref).  Test infrastructure only: they let the fixture
 * script set a system's box, positions and velocities to exact doubles and
 * read forces, energy and stress through the reference's own ForceFieldMD
 * boundary (ff_md.h:6-57), which its Python API does not expose.
 *
 * Every function takes the md.atoms Python object (ctypes.py_object).
 * Arrays are indexed by atom id (the order of the CFG file the atoms came
 * from), n x 3 row-major doubles; H is the 3 x 3 lower-triangular box,
 * row-major.  Return 0 on success, negative on a misuse.
 */
#include "atoms_md.h"
#include "dynamic_md.h"
#include "ff_md.h"

using namespace MAPP_NS;

namespace {

AtomsMD* atoms_of(PyObject* o)
{
    return o ? reinterpret_cast<AtomsMD::Object*>(o)->atoms : nullptr;
}

ForceFieldMD* ff_of(PyObject* o)
{
    return o ? reinterpret_cast<AtomsMD::Object*>(o)->ff : nullptr;
}

}  // namespace

extern "C" {

int mappg_ref_natms(PyObject* o)
{
    AtomsMD* a = atoms_of(o);
    return a ? a->natms : -1;
}

/* Box (update_H, atoms.cpp:187-194), then positions and (optionally)
 * velocities; the domain is reset for the new positions as atoms.do does. */
int mappg_ref_set_state(PyObject* o, const double* H, const double* x, const double* v)
{
    AtomsMD* a = atoms_of(o);
    if (!a) return -1;
    for (int i = 0; i < __dim__; i++)
        for (int j = 0; j < __dim__; j++) a->H[i][j] = H[3 * i + j];
    a->update_H();
    const int n = a->natms_lcl;
    const id_type* id = a->id->begin();
    type0* xp = a->x->begin();
    for (int i = 0; i < n; i++)
        for (int k = 0; k < 3; k++) xp[3 * i + k] = x[3 * (size_t)id[i] + k];
    if (v) {
        if (a->x_d->is_empty()) a->x_d->fill();
        type0* vp = a->x_d->begin();
        for (int i = 0; i < n; i++)
            for (int k = 0; k < 3; k++) vp[3 * i + k] = v[3 * (size_t)id[i] + k];
    }
    a->reset_domain();
    return 0;
}

int mappg_ref_get_state(PyObject* o, double* H, double* x, double* v)
{
    AtomsMD* a = atoms_of(o);
    if (!a) return -1;
    for (int i = 0; i < __dim__; i++)
        for (int j = 0; j < __dim__; j++) H[3 * i + j] = a->H[i][j];
    const int n = a->natms_lcl;
    const id_type* id = a->id->begin();
    const type0* xp = a->x->begin();
    const type0* vp = a->x_d->is_empty() ? nullptr : a->x_d->begin();
    for (int i = 0; i < n; i++)
        for (int k = 0; k < 3; k++) {
            if (x) x[3 * (size_t)id[i] + k] = xp[3 * i + k];
            if (v) v[3 * (size_t)id[i] + k] = vp ? vp[3 * i + k] : 0.0;
        }
    return 0;
}

/* One force call as MDNVT::run makes it (md_nvt.cpp:348 set-up, 387 call):
 * DynamicMD builds ghosts and the half list, ForceFieldMD::force_calc fills f,
 * pe and S_pe; value() is the energy-only pass (ff_eam.cpp:244-318).
 * res = [pe, S_pe (9, row-major), value()]. */
int mappg_ref_force(PyObject* o, double* f, double* res)
{
    AtomsMD* a = atoms_of(o);
    ForceFieldMD* ff = ff_of(o);
    if (!a || !ff) return -1;
    DynamicMD dyn(a, ff, false, {}, {a->x_d, a->x_dof}, {});
    dyn.init();
    ff->force_calc();
    const int n = a->natms_lcl;
    const id_type* id = a->id->begin();
    const type0* fp = ff->f->begin();
    for (int i = 0; i < n; i++)
        for (int k = 0; k < 3; k++) f[3 * (size_t)id[i] + k] = fp[3 * i + k];
    res[0] = a->pe;
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) res[1 + 3 * i + j] = a->S_pe[i][j];
    res[10] = ff->value();
    dyn.fin();
    return 0;
}

}  // extern "C"

extern "C" {

/* The minimizers' neighbour handling (NewDynamicMD<false,true>, used by
 * MinMDHandler for atoms-only relaxations, min_cg.h:106,265) in isolation:
 * initialise, move the atoms to x1 (by id), update as a line-search trial
 * does (MinMDHandler::F), then return derivative()'s energy and forces.
 * res = [pe after the update, value() after the update]. */
int mappg_ref_min_update_force(PyObject* o, const double* x1, double* f, double* res)
{
    AtomsMD* a = atoms_of(o);
    ForceFieldMD* ff = ff_of(o);
    if (!a || !ff) return -1;
    NewDynamicMD<false, true> dyn(a, ff, {}, {a->x_dof}, {});
    dyn.init();
    ff->derivative();
    const int n = a->natms_lcl;
    const id_type* id = a->id->begin();
    type0* xp = a->x->begin();
    for (int i = 0; i < n; i++)
        for (int k = 0; k < 3; k++) xp[3 * i + k] = x1[3 * (size_t)id[i] + k];
    dyn.update();
    res[1] = ff->value();
    res[0] = *ff->derivative();
    const type0* fp = ff->f->begin();
    id = a->id->begin();
    for (int i = 0; i < a->natms_lcl; i++)
        for (int k = 0; k < 3; k++) f[3 * (size_t)id[i] + k] = fp[3 * i + k];
    dyn.fin();
    return 0;
}

}  // extern "C"
