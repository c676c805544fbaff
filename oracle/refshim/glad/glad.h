// Stand-in for the OpenGL loader header: the one type CRender's entity header names.
// TEST INFRASTRUCTURE ONLY.
#pragma once
typedef unsigned int GLuint;
