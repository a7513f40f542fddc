// Engine-side access to a reference store's device copy (include/firepony_gb300_store.h).
#pragma once

#include <string>

#include "common.cuh"

struct fp_refstore;

namespace fpg {

// The store's device tables on `device`, uploading the image first if the store has no device copy; counts
// one more attached engine. nullptr with `err` set (and the status in `status`) on failure.
const DevRef *refstore_acquire(fp_refstore *store, int device, std::string &err, int &status);
// One engine fewer reads the store.
void refstore_release(fp_refstore *store);

}  // namespace fpg
