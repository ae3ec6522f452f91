/* Empty stand-in for the Windows SDK version header (targetver.h includes it). */
#pragma once
