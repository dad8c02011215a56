// libdvmh_gb: regular (non-distributed) variables of the program, dynamic
// arrays and the library initialisation of non-main translation units -- the
// calls cdvmh emits around regions and for C's allocation functions.
//
// Reference behaviour followed (rts/dvmh/...):
//   dvmh_init_lib_C              dvmh2.cpp:425-449   initialise once; later calls are ignored
//   dvmh_data_enter_C / _exit_C  dvmh2.cpp:1921-1979 a depth per address; at depth 0 the variable's
//                                runtime copy is dropped, read back first when saveFlag != 0
//   dvmh_variable_gen_header_C   dvmh2.cpp:1777-1859 the variable as data of rank 0 (a scalar) or of
//                                its array rank; the first axis of an incomplete array is sized from
//                                the bytes entered; a variable first seen while a region registers
//                                its data is entered implicitly and exits at the region's end
//                                (autoDataExit, dvmh2.cpp:1780-1784, 3128-3132)
//   dvmh_variable_get_header_C   dvmh2.cpp:1871-1882
//   dvmh_malloc_C ... _free_C    dvmh2.cpp:1981-2052 C allocation plus data enter / exit
//   dvmh_array_declare_C         dvmh2.cpp:501-523   an array whose first size is not known yet
//   dvmh_array_alloc_C           dvmh2.cpp:654-693   its storage: the first size from the bytes
//   dvmh_forget_header_          dvmh2.cpp:1750-1770 the descriptor goes out of scope
//   dvmh_get_own_element_addr_C  dvmh2.cpp:2957-2978 address of an element this process owns
//
// Where cdvmh emits them: converter_main.cpp:866-872 (globals), 973-980
// (dvmh_init_lib_C), 2568-2580 and 3000-3010, 3095-3100 (implicit data regions
// around loops and regions), 721-749 (declared arrays), 3332-3455 (own
// elements), 3385-3392 (dvmh_array_alloc_C); project_ctx.cpp:497-503 (the
// allocation functions).
//
// Here a scalar's rank-0 form is the runtime variable (Var) of its address --
// the object region registration, reductions and dvmh_get_device_addr_C
// already share -- and an array's form is an Array whose host copy is the
// program's own memory.
#include <cstdlib>
#include <cstring>
#include <map>
#include <vector>

#include "rt.h"

namespace dvmhgb {

namespace {

struct RegularVar {
    size_t size = 0;  // bytes entered (0: not known, an incomplete array)
    long depth = 0;
    Var *var = nullptr;    // rank-0 form
    Array *arr = nullptr;  // array form
};
std::map<const char *, RegularVar> regularVars;
std::vector<const char *> autoExit;  // entered implicitly by the current region

RegularVar *findRegular(const void *addr) {
    auto it = regularVars.find((const char *)addr);
    return it == regularVars.end() ? nullptr : &it->second;
}

size_t elemSize(DvmType ts) {
    if (ts > 0) return (size_t)ts;
    const size_t e = typeSize(-(int)ts);
    GB_CHECK(e > 0, "unknown data type %ld", (long)-ts);
    return e;
}

// drop the variable's runtime forms (after reading them back when `save`)
void dropForms(const char *addr, RegularVar &rv, bool save) {
    if (rv.arr) {
        GB_CHECK(!(st.curRegion && rv.arr->regMark == st.curRegion),
                 "regular array at %p leaves its data region inside a region that uses it", (const void *)addr);
        if (save) ensureHostActual(rv.arr);
        arrayRelease(rv.arr);
        rv.arr = nullptr;
    }
    if (rv.var) {
        Var *v = rv.var;
        if (save && !v->hostActual) {
            queueFlush();
            varD2H(v);
            v->hostActual = true;
        }
        varDrop(v);
        rv.var = nullptr;
    }
}

}  // namespace

bool regularActual(const void *addr, bool toHost) {
    RegularVar *rv = findRegular(addr);
    if (!rv || !rv->arr) return false;
    if (toHost) {
        ensureHostActual(rv->arr);
    } else {
        rv->arr->hostActual = true;
        rv->arr->devActual = false;
    }
    return true;
}

Var *regularVarOfHeader(const void *p) {
    for (auto &kv : regularVars)
        if (kv.second.var && (const void *)kv.second.var->hdr == p) return kv.second.var;
    return nullptr;
}

void regularRegionEnd() {
    std::vector<const char *> pending;
    pending.swap(autoExit);
    for (const char *a : pending) dvmh_data_exit_C(a, 1);
}

}  // namespace dvmhgb

using namespace dvmhgb;

extern "C" {

void dvmh_init_lib_C(DvmType flags) {
    // a library's translation unit: initialise unless the program already did
    if (!st.inited) dvmh_init_C(flags, nullptr, nullptr);
}

void dvmh_init_lib_(const DvmType *pFlags) {
    GB_CHECK(pFlags, "NULL flags passed to dvmh_init_lib_");
    dvmh_init_lib_C(*pFlags);
}

void dvmh_data_enter_C(const void *addr, DvmType size) {
    GB_CHECK(st.inited, "LibDVMH is not initialized");
    GB_CHECK(size >= 0, "Negative size is passed to dvmh_data_enter");
    GB_CHECK(addr, "NULL pointer is passed to dvmh_data_enter");
    RegularVar &rv = regularVars[(const char *)addr];
    if ((size_t)size > rv.size) rv.size = (size_t)size;
    rv.depth++;
    logmsg(LOG_TRACE, "variable at %p (%ld bytes) entered a data region, depth %ld", addr, (long)size, rv.depth);
}

void dvmh_data_enter_(const void *addr, const DvmType *pSize) {
    GB_CHECK(pSize, "NULL size passed to dvmh_data_enter_");
    dvmh_data_enter_C(addr, *pSize);
}

void dvmh_data_exit_C(const void *addr, DvmType saveFlag) {
    GB_CHECK(st.inited, "LibDVMH is not initialized");
    GB_CHECK(addr, "NULL pointer is passed to dvmh_data_exit");
    RegularVar *rv = findRegular(addr);
    GB_CHECK(rv, "Unknown variable is passed to dvmh_data_exit");
    GB_CHECK(rv->depth > 0, "Data region enter/exit imbalance detected");
    rv->depth--;
    if (rv->depth > 0) return;
    dropForms((const char *)addr, *rv, saveFlag != 0);
    regularVars.erase((const char *)addr);
}

void dvmh_data_exit_(const void *addr, const DvmType *pSaveFlag) {
    GB_CHECK(pSaveFlag, "NULL flag passed to dvmh_data_exit_");
    dvmh_data_exit_C(addr, *pSaveFlag);
}

DvmType *dvmh_variable_gen_header_C(const void *addr, DvmType rank, DvmType typeSize, ...) {
    GB_CHECK(st.inited, "LibDVMH is not initialized");
    GB_CHECK(addr, "NULL pointer is passed to dvmh_variable_gen_header");
    GB_CHECK(rank >= 0 && rank <= MAXR, "Invalid rank is passed to dvmh_variable_gen_header");
    const size_t esize = elemSize(typeSize);
    long ext[MAXR] = {};
    va_list ap;
    va_start(ap, typeSize);
    for (int i = 0; i < rank; i++) ext[i] = (long)va_arg(ap, DvmType);
    va_end(ap);
    RegularVar *rv = findRegular(addr);
    if (!rv) {
        // first seen while a region (or a loop outside regions) registers its data:
        // entered implicitly until that region or loop ends
        GB_CHECK((st.curRegion && !st.curRegion->started) || (!st.curRegion && st.curLoop),
                 "Unknown regular variable at %p", addr);
        dvmh_data_enter_C(addr, 0);
        autoExit.push_back((const char *)addr);
        rv = findRegular(addr);
    }
    size_t rest = esize;
    for (int i = 1; i < rank; i++) {
        GB_CHECK(ext[i] > 0, "non-positive size %ld of a regular array on axis %d", ext[i], i + 1);
        rest *= (size_t)ext[i];
    }
    const size_t bytes = rank > 0 ? std::max(rv->size, rest * (size_t)std::max(ext[0], 0L)) : esize;
    if (bytes > rv->size) rv->size = bytes;
    if (rank == 0) {
        if (!rv->var) rv->var = varGet(addr, esize);
        GB_CHECK(rv->var->size == esize, "Regular variable configuration has been changed");
        rv->var->hdr[0] = (DvmType)rv->var;
        return rv->var->hdr;
    }
    const long first = (long)(rv->size / rest);  // the first axis from the bytes entered
    GB_CHECK(first > 0, "regular array at %p has no elements", addr);
    if (rv->arr) {
        Array *a = rv->arr;
        bool same = a->rank == rank && a->esize == esize && a->ext[0] == first;
        for (int i = 1; i < rank; i++) same = same && a->ext[i] == ext[i];
        GB_CHECK(same, "Regular variable configuration has been changed");
        return a->ownHdr;
    }
    GB_CHECK(!st.curRegion || !st.curRegion->started,
             "regular array at %p first used after its region started executing", addr);
    long sizes[MAXR], zero[MAXR] = {};
    sizes[0] = first;
    for (int i = 1; i < rank; i++) sizes[i] = ext[i];
    Array *a = arrayNew(nullptr, (int)rank, typeSize, sizes, zero, zero);
    arrayAttachHost(a, (char *)addr);
    alignIdentity(a->align, a, a->rank);
    rv->arr = a;
    return a->ownHdr;
}

DvmType *dvmh_variable_get_header_C(const void *addr) {
    GB_CHECK(st.inited, "LibDVMH is not initialized");
    GB_CHECK(addr, "NULL pointer is passed to dvmh_variable_get_header");
    RegularVar *rv = findRegular(addr);
    GB_CHECK(rv && (rv->arr || rv->var), "Unknown variable is passed to dvmh_variable_get_header");
    return rv->arr ? rv->arr->ownHdr : rv->var->hdr;
}

void *dvmh_malloc_C(size_t size) {
    void *res = malloc(size);
    if (res) {
        GB_INTERNAL(!findRegular(res), "Variable tracking error");
        dvmh_data_enter_C(res, (DvmType)size);
    }
    return res;
}

void *dvmh_calloc_C(size_t nmemb, size_t size) {
    void *res = calloc(nmemb, size);
    if (res) {
        GB_INTERNAL(!findRegular(res), "Variable tracking error");
        dvmh_data_enter_C(res, (DvmType)(nmemb * size));
    }
    return res;
}

void *dvmh_realloc_C(void *ptr, size_t size) {
    if (ptr && findRegular(ptr)) dvmh_data_exit_C(ptr, 1);  // the current value moves with the block
    GB_INTERNAL(!ptr || !findRegular(ptr), "Dynamically allocated variable enter/exit imbalance");
    void *res = realloc(ptr, size);
    if (res) {
        GB_INTERNAL(!findRegular(res), "Variable tracking error");
        dvmh_data_enter_C(res, (DvmType)size);
    }
    return res;
}

char *dvmh_strdup_C(const char *s) {
    char *res = strdup(s);
    if (res) {
        GB_INTERNAL(!findRegular(res), "Variable tracking error");
        dvmh_data_enter_C(res, (DvmType)(strlen(res) + 1));
    }
    return res;
}

void dvmh_free_C(void *ptr) {
    if (ptr && findRegular(ptr)) dvmh_data_exit_C(ptr, 0);
    GB_INTERNAL(!ptr || !findRegular(ptr), "Dynamically allocated variable enter/exit imbalance");
    free(ptr);
}

void dvmh_array_declare_C(DvmType dvmDesc[], DvmType rank, DvmType typeSize, ...) {
    GB_CHECK(st.inited, "LibDVMH is not initialized");
    GB_CHECK(!st.curRegion && !st.curLoop, "dvmh_array_declare is not allowed in a region or a parallel loop");
    GB_CHECK(dvmDesc, "NULL descriptor passed to dvmh_array_declare");
    GB_CHECK(rank > 0 && rank <= MAXR, "array rank must be in 1..%d (got %ld)", MAXR, (long)rank);
    (void)elemSize(typeSize);
    Decl *d = new Decl();
    d->rank = (int)rank;
    d->typeSize = typeSize;
    va_list ap;
    va_start(ap, typeSize);
    for (int i = 0; i < d->rank; i++) {
        d->ext[i] = (long)va_arg(ap, DvmType);
        d->shLo[i] = (long)va_arg(ap, DvmType);
        d->shHi[i] = (long)va_arg(ap, DvmType);
    }
    va_end(ap);
    for (int i = 0; i < d->rank; i++) {
        GB_CHECK(i == 0 || d->ext[i] > 0, "Negative size of array on axis %d: %ld", i + 1, d->ext[i]);
        GB_CHECK(d->shLo[i] >= 0, "Negative lower shadow width on axis %d: %ld", i + 1, d->shLo[i]);
        GB_CHECK(d->shHi[i] >= 0, "Negative upper shadow width on axis %d: %ld", i + 1, d->shHi[i]);
    }
    trackObj(d);
    dvmDesc[0] = (DvmType)d;
}

void dvmh_array_alloc_C(DvmType dvmDesc[], DvmType byteCount) {
    GB_CHECK(st.inited, "LibDVMH is not initialized");
    GB_CHECK(!st.curRegion && !st.curLoop, "dvmh_array_alloc is not allowed in a region or a parallel loop");
    GB_CHECK(dvmDesc, "NULL descriptor passed to dvmh_array_alloc");
    Obj *o = (Obj *)dvmDesc[0];
    GB_CHECK(o, "NULL object is passed to dvmh_array_alloc");
    GB_CHECK(!isLive(o, K_ARRAY),
             "Either DVM-array usage violation or memory leak detected. Consider using another DVM-array variable "
             "or freeing dynamically allocated memory beforehand.");
    GB_CHECK(isLive(o, K_DECL), "Only declared array pointer can be passed to dvmh_array_alloc");
    Decl *d = (Decl *)o;
    const size_t esize = elemSize(d->typeSize);
    size_t rest = esize;
    for (int i = 1; i < d->rank; i++) rest *= (size_t)d->ext[i];
    GB_CHECK(byteCount > 0 && (size_t)byteCount % rest == 0,
             "Allocation amount (%ld) must be exact, i.e. a product of all the array's dimension sizes",
             (long)byteCount);
    long ext[MAXR];
    memcpy(ext, d->ext, sizeof ext);
    ext[0] = (long)((size_t)byteCount / rest);
    const int rank = d->rank;
    const DvmType typeSize = d->typeSize;
    long shLo[MAXR], shHi[MAXR];
    memcpy(shLo, d->shLo, sizeof shLo);
    memcpy(shHi, d->shHi, sizeof shHi);
    untrackObj(d);
    delete d;
    arrayNew(dvmDesc, rank, typeSize, ext, shLo, shHi);
}

void dvmh_forget_header_(DvmType dvmDesc[]) {
    GB_CHECK(st.inited, "LibDVMH is not initialized");
    GB_CHECK(dvmDesc, "NULL descriptor passed to dvmh_forget_header");
    Obj *o = (Obj *)dvmDesc[0];
    if (o) {
        if (isLive(o, K_ARRAY)) {
            // the program's descriptor goes out of scope; the array itself stays (the
            // reference removes the header and keeps the data), known by its own header
            Array *a = (Array *)o;
            GB_CHECK(a->desc == dvmDesc,
                     "Memory leak detected. Consider freeing dynamically allocated memory beforehand.");
            arrayRetarget(a, a->ownHdr);
        } else if (isLive(o, K_DECL)) {
            untrackObj(o);
            delete (Decl *)o;
        } else {
            GB_CHECK(false, "Only array can be passed to dvmh_forget_header");
        }
    }
    dvmDesc[0] = 0;
}

void *dvmh_get_own_element_addr_C(const DvmType dvmDesc[], DvmType rank, ...) {
    GB_CHECK(st.inited, "LibDVMH is not initialized");
    Array *a = arrayOf(dvmDesc, "dvmh_get_own_element_addr");
    GB_CHECK(a->rank == rank, "Rank in every indexing expression must be the same as in declaration of the variable");
    va_list ap;
    va_start(ap, rank);
    long lin = 0;
    bool own = true;
    for (int i = 0; i < a->rank; i++) {
        const long idx = (long)va_arg(ap, DvmType);
        own = own && idx >= 0 && idx < a->ext[i];
        lin += idx * a->hstride[i];
    }
    va_end(ap);
    // one process owns every element of the index space
    return own ? (void *)(a->host + lin * (long)a->esize) : nullptr;
}

}  // extern "C"

// ---------------------------------------------------------------- module initialisers
// (rts/dvmh/dvmh_rts.cpp:1530-1559: a list of the translation units' init and
// finish functions; init runs at runtime initialisation, or at once when the
// runtime is already up -- a library loaded later)

DvmhModuleInitializer *DvmhModuleInitializer::head = nullptr;

DvmhModuleInitializer::DvmhModuleInitializer(void (*fInit)(), void (*fFinish)()) {
    next = head;
    head = this;
    funcInit = fInit;
    funcFinish = fFinish;
    if (st.inited && funcInit) funcInit();
}

void DvmhModuleInitializer::executeInit() {
    for (DvmhModuleInitializer *cur = head; cur; cur = cur->next)
        if (cur->funcInit) cur->funcInit();
}

void DvmhModuleInitializer::executeFinish() {
    for (DvmhModuleInitializer *cur = head; cur; cur = cur->next)
        if (cur->funcFinish) cur->funcFinish();
}
