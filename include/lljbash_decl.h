/*
 * Symbol-prefix and struct-declaration helpers shared by every public header.
 * Replaces the reference's include/lljbash_decl.h:1-21 with the same macro names and
 * meaning, so that every C-visible name is exported as LLJBASH_<Name> and C++ builds
 * get default member values while C builds get plain structs.
 */
#pragma once

#ifndef LLJBASH_DECL
#define LLJBASH_DECL(name) LLJBASH_##name
#endif

#ifndef LLJBASH_DEFAULT_VALUE
#ifdef __cplusplus
#define LLJBASH_DEFAULT_VALUE(a) = a
#else
#define LLJBASH_DEFAULT_VALUE(a)
#endif
#endif

#ifndef LLJBASH_STRUCT_TYPEDEF
#ifndef __cplusplus
#define LLJBASH_STRUCT_TYPEDEF(s) typedef struct s s
#else
#define LLJBASH_STRUCT_TYPEDEF(s)
#endif
#endif

#ifndef LLJBASH_NULL
#ifdef __cplusplus
#define LLJBASH_NULL nullptr
#else
#define LLJBASH_NULL 0
#endif
#endif
