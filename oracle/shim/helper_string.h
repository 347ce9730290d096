/* Project-written stand-in for the CUDA-samples header (struct.h:6). */
#pragma once
int getCmdLineArgumentInt(int argc, const char **argv, const char *name);
bool getCmdLineArgumentString(int argc, const char **argv, const char *name, char **value);
