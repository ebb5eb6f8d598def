/* Forced-include prelude for compiling the PD reference sources out of tree.
 *
 * PD's mmlib/exception.h guards itself with __EXCEPTION_H, the same macro that
 * libstdc++'s <bits/exception.h> uses, so whichever comes second is silently
 * dropped.  This prelude pulls in the standard header first, clears the macro
 * and then includes PD's header so both sets of declarations are seen.  It
 * also supplies the standard headers that PD forgets to include.  Nothing in
 * the reference tree is modified or copied.
 */
#ifndef PDGPU_REF_PRELUDE_H
#define PDGPU_REF_PRELUDE_H
#include <climits>
#include <typeinfo>
#include <cstring>
#include <cstdio>
#include <cstdlib>
#include <algorithm>
#include <exception>
#include <iostream>
#include <fstream>
#include <vector>
#include <string>
#undef __EXCEPTION_H
#include "mmlib/global.h"
#endif
