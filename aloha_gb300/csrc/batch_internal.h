// batch_internal.h -- context accessors shared by api.cpp and batch.cpp.
#pragma once

#include "internal.h"

namespace aloha {

int ctx_fail(aloha_ctx* c, int code, const char* fmt, ...);
int ctx_device(const aloha_ctx* c);
int ctx_num_sms(const aloha_ctx* c);
int ctx_n_tf(const aloha_ctx* c);
void ctx_view_size(const aloha_ctx* c, int view, int* w, int* h);
void ctx_frame_args(aloha_ctx* c, FrameArgs* a);
int ctx_prepare_view(aloha_ctx* c, int view, cudaStream_t s);
void ctx_mark_samples(aloha_ctx* c);
bool ctx_is_device_pointer(const void* p);
// True for device (or managed) memory that the given device can use as its own:
// device memory of that device, or managed memory.
bool device_pointer_on(const void* p, int device);

}  // namespace aloha
