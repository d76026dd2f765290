/* Stand-in (oracle harness only): the GL types the reference's class headers name. */
#pragma once
typedef unsigned int GLuint;
typedef int GLint;
