/* Minimal stand-in for the MSVC <tchar.h> (stdafx.h includes it). */
#pragma once
typedef char _TCHAR;
#define _tmain main
