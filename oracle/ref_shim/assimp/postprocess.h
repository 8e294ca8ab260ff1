#pragma once
enum aiPostProcessSteps { aiProcessPreset_TargetRealtime_MaxQuality = 0 };
