// les_io.h -- handle access that les_api.cu gives the file readers and writers.
#pragma once

#include "../../include/les_gpu.h"

int les_handle_dims(const les_handle *h, int *im, int *jm, int *km);
// Records msg as the handle's last error and returns code.
int les_handle_fail(les_handle *h, int code, const char *msg);
