// pt_abi_guard.h - no C++ exception leaves a C entry point of the library.
// Entry points that allocate on the host are function-try-blocks whose
// handler returns pt_abi_status(obj): PT_ERR_OOM for an allocation failure,
// PT_ERR_INVALID_ARG (with the exception's text) for anything else, the
// message stored as the object's last error when there is an object.
#pragma once

#include <exception>
#include <new>
#include <string>

#include "../../include/pt.h"

// the status of the exception being handled; its text into *message (no throw)
inline int pt_abi_current_status(std::string* message) noexcept {
    int code = PT_ERR_INVALID_ARG;
    const char* text = "unexpected error";
    try {
        throw;
    } catch (const std::bad_alloc&) {
        code = PT_ERR_OOM;
        text = "out of host memory";
    } catch (const std::exception& e) {
        text = e.what();
    } catch (...) {
    }
    if (message) {
        try {
            *message = text;
        } catch (...) {
        }
    }
    return code;
}

// inside a catch handler: the status, with the message kept in obj->error
template <class T>
int pt_abi_status(T* obj) noexcept {
    return pt_abi_current_status(obj ? &obj->error : nullptr);
}
