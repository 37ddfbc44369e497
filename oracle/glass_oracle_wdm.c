/* WDM restatement: filled in below. */
