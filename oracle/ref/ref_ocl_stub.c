/* OpenCL-less stand-in for the reference's tay/ocl_wrappers.c.
 *
 * Test infrastructure only.  The oracle runs the reference's CPU path; the OpenCL
 * device path is never enabled (tay_switch_to_ocl is not called), but tay/ocl.c and
 * tay/ocl_grid.c still reference the wrapper functions declared in tay/ocl.h:81-96, and
 * tay/state.c:38 calls ocl_release_context unconditionally.  Every wrapper reports
 * failure (0 / NULL, the reference's error convention, tay/ocl_wrappers.c:8-12) and
 * touches no device. */
#include "ocl.h"
#include "state.h"

int ocl_init_context(TayState *state, OclDevice *device) {
    (void)state;
    device->enabled = 0;
    return 0;
}

void ocl_release_context(OclDevice *device) {
    device->enabled = 0;
}

void *ocl_create_program(TayState *state, OclText *text) {
    (void)state; (void)text;
    return 0;
}

void *ocl_create_kernel(TayState *state, char *name) {
    (void)state; (void)name;
    return 0;
}

void *ocl_create_read_write_buffer(TayState *state, unsigned size) {
    (void)state; (void)size;
    return 0;
}

void *ocl_create_read_only_buffer(TayState *state, unsigned size) {
    (void)state; (void)size;
    return 0;
}

int ocl_read_buffer_blocking(TayState *state, void *ocl_buffer, void *buffer, unsigned size) {
    (void)state; (void)ocl_buffer; (void)buffer; (void)size;
    return 0;
}

int ocl_read_buffer_non_blocking(TayState *state, void *ocl_buffer, void *buffer, unsigned size) {
    (void)state; (void)ocl_buffer; (void)buffer; (void)size;
    return 0;
}

int ocl_write_buffer_blocking(TayState *state, void *ocl_buffer, void *buffer, unsigned size) {
    (void)state; (void)ocl_buffer; (void)buffer; (void)size;
    return 0;
}

int ocl_write_buffer_non_blocking(TayState *state, void *ocl_buffer, void *buffer, unsigned size) {
    (void)state; (void)ocl_buffer; (void)buffer; (void)size;
    return 0;
}

int ocl_fill_buffer(TayState *state, void *buffer, unsigned size, int pattern) {
    (void)state; (void)buffer; (void)size; (void)pattern;
    return 0;
}

int ocl_set_buffer_kernel_arg(TayState *state, unsigned arg_index, void *kernel, void **buffer) {
    (void)state; (void)arg_index; (void)kernel; (void)buffer;
    return 0;
}

int ocl_set_value_kernel_arg(TayState *state, unsigned arg_index, void *kernel, void *value, unsigned value_size) {
    (void)state; (void)arg_index; (void)kernel; (void)value; (void)value_size;
    return 0;
}

int ocl_run_kernel(TayState *state, void *kernel, unsigned global_size, unsigned local_size) {
    (void)state; (void)kernel; (void)global_size; (void)local_size;
    return 0;
}

int ocl_finish(TayState *state) {
    (void)state;
    return 0;
}

void ocl_release_program(void *program) {
    (void)program;
}

void ocl_release_buffer(void *buffer) {
    (void)buffer;
}
