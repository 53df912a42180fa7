/* Intrusive reference counting for the vr shim (test infrastructure only). */
#ifndef GRIDRT_SHIM_VR_REF_COUNTING_H
#define GRIDRT_SHIM_VR_REF_COUNTING_H

#include <vr/common.h>

namespace vr {

class RefCounted {
public:
    RefCounted() : _refs(0) {}
    void ref() const { ++_refs; }
    void unref() const {
        if (--_refs <= 0) delete this;
    }
    int refCount() const { return _refs; }

protected:
    virtual ~RefCounted() {}

private:
    mutable int _refs;
};

template <typename T>
class ref_ptr {
public:
    ref_ptr() : _p(nullptr) {}
    ref_ptr(T* p) : _p(p) { if (_p) _p->ref(); }
    ref_ptr(const ref_ptr& o) : _p(o._p) { if (_p) _p->ref(); }
    ~ref_ptr() { if (_p) _p->unref(); }
    ref_ptr& operator=(T* p) {
        if (p) p->ref();
        if (_p) _p->unref();
        _p = p;
        return *this;
    }
    ref_ptr& operator=(const ref_ptr& o) { return *this = o._p; }
    T* get() const { return _p; }
    T* operator->() const { return _p; }
    T& operator*() const { return *_p; }
    bool valid() const { return _p != nullptr; }

private:
    T* _p;
};

}  // namespace vr

#endif
